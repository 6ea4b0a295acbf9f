import importlib
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _ensure_oracle():
    lib = os.path.join(ROOT, "oracle", "_build", "libpd_oracle.so")
    src = [os.path.join(ROOT, "oracle", f) for f in ("pd_oracle.c", "pd_oracle.h")]
    if not os.path.exists(lib) or any(os.path.getmtime(s) > os.path.getmtime(lib) for s in src):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)


_ensure_oracle()


@pytest.fixture(scope="session")
def pdg():
    m = importlib.import_module("2d_pd_gpu_gb300")
    if not os.path.exists(m.native.LIB_PATH):
        importlib.import_module("2d_pd_gpu_gb300.build").build()
    return m


@pytest.fixture(scope="session")
def po():
    import pd_oracle

    return pd_oracle


@pytest.fixture(scope="session")
def hassa():
    return dict(np.load(os.path.join(GOLDEN, "hassa_ref.npz")))


@pytest.fixture(scope="session")
def plate30_ref():
    return dict(np.load(os.path.join(GOLDEN, "plate30_ref.npz")))


def normwise(a, ref):
    """max|a - ref| / max|ref| (elementwise relative error is meaningless where
    the reference is rounding noise, e.g. interior velocities of ~1e-19)."""
    den = np.abs(ref).max()
    return float(np.abs(a - ref).max() / (den if den > 0 else 1.0))


def hassa_oracle(po, h, n1n2_zero=True):
    """The oracle on the reference's Hassa problem (its main's parameters)."""
    n = h["x"].shape[0]
    bc = np.zeros(n, np.uint8)
    bc[h["top"]] = 1
    bc[h["bottom"]] = 2
    dx, hor, E, nu, rho, dt = h["params"]
    return po.OracleSim(h["x"], h["vol"], h["row_ptr"], h["col"], E=E, nu=nu, rho=rho, dt=dt, s_c=0.0, bc=bc,
                        group_kind=np.array([po.BC_VELOCITY, po.BC_FIXED], np.int32),
                        group_val=np.array([[0.0, 5.0], [0.0, 0.0]]))


def plate_oracle(po, p, s_c=None, families=None, k_hg=None):
    rp, col = families if families is not None else po.build_families(p.x, p.cutoff, p.cracks)
    return po.OracleSim(p.x, p.vol, rp, col, E=p.material.E, nu=p.material.nu, rho=p.material.rho, dt=p.dt,
                        s_c=p.material.s_c if s_c is None else s_c, k_hg=p.k_hg if k_hg is None else k_hg,
                        damage_fail=p.damage_fail, bc=p.group_of, group_kind=p.group_kind, group_val=p.group_val)
