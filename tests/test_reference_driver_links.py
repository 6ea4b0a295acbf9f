"""The reference's own GPU driver (src/main.cu), unmodified, compiles and
links against the C++ drop-in when include/compat shadows its mechanics.cuh.

Only where the reference checkout exists (it is not on the GPU machine);
compile and link only -- running it needs the GPU.  The stub mpi/parmetis/
Eigen headers are the oracle's (the reference's driver includes them; a
maintainer's machine has the real ones).
"""
import os
import subprocess

import pd_oracle
import pytest

from conftest import ROOT

REF = pd_oracle.reference_dir()  # PD_REFERENCE_DIR, or the checkout oracle/_ref was built from


@pytest.mark.skipif(not REF or not os.path.exists(os.path.join(REF, "src", "main.cu")),
                    reason="reference checkout absent (set PD_REFERENCE_DIR)")
def test_reference_main_cu_links_against_dropin(pdg, tmp_path):
    libdir = os.path.dirname(pdg.native.LIB_PATH)
    exe = str(tmp_path / "ref_main_on_gb300")
    cmd = ["nvcc", "-std=c++17", "-w", "-x", "cu",
           f"-I{os.path.join(ROOT, 'include', 'compat')}", f"-I{os.path.join(ROOT, 'include')}",
           f"-I{os.path.join(ROOT, 'oracle', 'ref_stubs')}", f"-I{os.path.join(REF, 'include')}",
           os.path.join(REF, "src", "main.cu"), "-o", exe, f"-L{libdir}", "-lpd_dropin", "-lpd_gb300",
           f"-Xlinker", f"-rpath={libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    # the hot path resolves to the drop-in (undefined in the driver, provided by libpd_dropin.so)
    assert any("U compute_velocity_GPU_host(" in l for l in out.splitlines())
