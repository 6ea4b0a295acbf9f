"""Mazars damage on the GPU (pd_mazars_*, csrc/pd_mazars.cu) against the
reference's computeDamageStatus (tests/golden/mazars_ref.npz: the Hassa mesh
at two imposed displacement fields, classic and n1 = n2 = 10 weights) and
against the oracle restatement."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_oracle_golden import MZ_TOL, mazars_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mz():
    return dict(np.load(os.path.join(GOLDEN, "mazars_ref.npz")))


def _ctx(pdg, h, w):
    dx, hor, E, nu, rho, dt = h["params"]
    ctx = pdg.native.Context(pdg.default_params(E=E, nu=nu, rho=rho, dt=dt, s_c=0.0, n1=w, n2=w,
                                                weight_len=hor * dx))
    ctx.set_particles(h["x"], h["vol"])
    ctx.set_families(h["row_ptr"], h["col"])
    return ctx


@pytest.mark.parametrize("tag,w", [("c", 0.0), ("b", 10.0)])
def test_gpu_mazars_matches_reference(pdg, hassa, mz, tag, w):
    ctx = _ctx(pdg, hassa, w)
    k0 = float(mz["kappa0"])
    ctx.mazars_init(kappa0=k0)
    ctx.set_state(u=mz["u1"])
    ctx.mazars_update()
    thr, bd, st = ctx.mazars()
    assert int((thr > k0).sum()) == int(mz[f"{tag}_updated1"])
    assert np.abs(st - mz[f"{tag}_st1"]).max() < MZ_TOL
    ctx.set_state(u=mz["u2"])
    ctx.mazars_update()
    thr, bd, st = ctx.mazars()
    assert np.abs(st - mz[f"{tag}_st2"]).max() < MZ_TOL
    assert np.abs(thr - mz[f"{tag}_thr2"]).max() < MZ_TOL * np.abs(mz[f"{tag}_thr2"]).max()
    assert np.abs(bd - mz[f"{tag}_bd2"]).max() < MZ_TOL


def test_gpu_mazars_classic_strain_bit_exact_vs_oracle(pdg, po, hassa, mz):
    """Classic weights: the equivalent strain (the thresholds) is the oracle's
    bit for bit (same FP64 operation sequence); the damage differs only by
    CUDA's exp in the last bits."""
    ctx = _ctx(pdg, hassa, 0.0)
    sim = mazars_oracle(po, hassa, 0.0)
    k0 = float(mz["kappa0"])
    ctx.mazars_init(kappa0=k0)
    nnz = int(hassa["row_ptr"][-1])
    thr, bd = np.full(nnz, k0), np.zeros(nnz)
    for lv in (1, 2):
        ctx.set_state(u=mz[f"u{lv}"])
        ctx.mazars_update()
        sim.u[:] = mz[f"u{lv}"]
        st = sim.mazars(thr, bd, k0)
        gthr, gbd, gst = ctx.mazars()
        assert np.array_equal(gthr, thr)
        assert np.abs(gbd - bd).max() < 1e-14 and np.abs(gst - st).max() < 1e-14


def test_gpu_mazars_set_get_and_checkpoint(pdg, hassa, mz):
    ctx = _ctx(pdg, hassa, 0.0)
    k0 = float(mz["kappa0"])
    ctx.mazars_init(kappa0=k0)
    ctx.set_state(u=mz["u1"])
    ctx.mazars_update()
    thr, bd, st = ctx.mazars()
    blob = ctx.checkpoint()
    other = _ctx(pdg, hassa, 0.0)  # no Mazars history yet: the blob brings it
    other.restore(blob)
    t2, b2, s2 = other.mazars()
    assert np.array_equal(t2, thr) and np.array_equal(b2, bd) and np.array_equal(s2, st)
    third = _ctx(pdg, hassa, 0.0)
    third.mazars_init(kappa0=k0)
    third.mazars_set(threshold=thr, bond_damage=bd)
    t3, b3, s3 = third.mazars()
    assert np.array_equal(t3, thr) and np.array_equal(b3, bd) and np.abs(s3 - st).max() == 0.0


def test_gpu_mazars_rejects_mixed(pdg):
    p = pdg.plates.make_plate(16, seed=1)
    c = p.context(precision=pdg.native.PD_MIXED)
    with pytest.raises(pdg.PdError):
        c.mazars_init()
