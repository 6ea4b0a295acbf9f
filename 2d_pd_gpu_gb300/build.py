"""Build the native libraries in-tree (no cmake, no pip install).

    python -m 2d_pd_gpu_gb300.build      (or __graft_entry__.build())

produces 2d_pd_gpu_gb300/_build/libpd_gb300.so (CUDA kernels + C ABI, sm_103a
only), 2d_pd_gpu_gb300/_build/libpd_dropin.so (the C++ drop-in with the
reference's function names, linked against libpd_gb300.so) and
2d_pd_gpu_gb300/_build/pd_hassa_timing (the drop-in timed on the reference's
own published problem, see csrc/pd_hassa_timing.cpp).  Translation
units compile in parallel.  Files whose results must match the FP64 oracle
bit-for-bit are compiled with --fmad=false (only explicit fma() fuses).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                      f"-I{INCLUDE}", f"-I{CSRC}", "-Xptxas", "-warn-spills"]

# (source, extra flags)
CUDA_UNITS = [
    ("pd_family.cu", ["--fmad=false"]),
    ("pd_fp64.cu", ["--fmad=false"]),
    ("pd_bondassoc.cu", ["--fmad=false"]),
    ("pd_mixed.cu", []),
    ("pd_noalloc.cu", ["--fmad=false"]),
    ("pd_mazars.cu", ["--fmad=false"]),
    ("pd_order.cu", []),
    ("pd_probe.cu", []),
    ("pd_api.cu", []),
]
DROPIN_UNITS = ["pd_dropin.cpp"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, h) for h in ("pd_internal.h", "pd_walk.cuh", "pd_batch.cuh", "pd_stage.cuh")] + \
        [os.path.join(INCLUDE, "pd_gb300.h")]
    objs, jobs = [], []
    for src, extra in CUDA_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nv] + NVCC_COMMON + extra + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    lib = os.path.join(OUT, "libpd_gb300.so")
    if force or jobs or _stale(lib, objs):
        _run([nv] + ARCH + ["-shared", "-o", lib] + objs)
    # C++ drop-in (host only), linked against libpd_gb300.so with an rpath to it
    dsrc = [os.path.join(CSRC, u) for u in DROPIN_UNITS if os.path.exists(os.path.join(CSRC, u))]
    if dsrc:
        dlib = os.path.join(OUT, "libpd_dropin.so")
        dh = [os.path.join(INCLUDE, "pd_dropin.h")]
        if force or _stale(dlib, dsrc + dh + [lib]):
            _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-I{INCLUDE}", "-o", dlib] + dsrc +
                 [f"-L{OUT}", "-lpd_gb300", "-Wl,-rpath,$ORIGIN"])
        # the timing driver for the reference's published problem (bench.py's bond-associated leg)
        tsrc = os.path.join(CSRC, "pd_hassa_timing.cpp")
        texe = os.path.join(OUT, "pd_hassa_timing")
        if force or _stale(texe, [tsrc, dlib] + dh + [os.path.join(INCLUDE, "pd_gb300.h")]):
            _run(["g++", "-O2", "-std=c++17", f"-I{INCLUDE}", tsrc, "-o", texe, f"-L{OUT}", "-lpd_dropin",
                  "-lpd_gb300", "-Wl,-rpath,$ORIGIN"])
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
