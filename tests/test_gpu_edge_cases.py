"""Edge cases of the device path against the oracle: empty and tiny
problems, partial SELL chunks and blocks, ragged families (holes), the
largest families the layout takes, and family overflow."""
import dataclasses

import numpy as np
import pytest

from conftest import normwise, plate_oracle
from test_gpu_fp64_parity import _assert_same

pytestmark = pytest.mark.gpu


def _subset(p, keep):
    keep = np.asarray(keep)
    return dataclasses.replace(p, x=np.ascontiguousarray(p.x[keep]), vol=np.ascontiguousarray(p.vol[keep]),
                               group_of=np.ascontiguousarray(p.group_of[keep]))


@pytest.mark.parametrize("precision", [0, 1])
def test_empty_problem(pdg, precision):
    ctx = pdg.native.Context(pdg.default_params(precision=precision))
    ctx.set_particles(np.zeros((0, 2)), np.zeros(0))
    ctx.build_families(1.0)
    ctx.step(3)
    u, v, f = ctx.state()
    assert u.shape == (0, 2) and ctx.nnz == 0 and ctx.counters()["steps"] == 3


@pytest.mark.parametrize("n", [1, 2, 31, 33, 35, 257])
def test_tiny_and_partial_chunks_bit_exact(pdg, po, n):
    """n not a multiple of the 32-particle chunk or the 256-particle block."""
    p = _subset(pdg.plates.make_plate(20, seed=6, crack="centre-half"), np.arange(n))
    p.material.s_c = 2e-4
    ctx = p.context()
    sim = plate_oracle(po, p)
    ctx.step(15)
    sim.step(15)
    _assert_same(ctx, sim)
    m = p.context(precision=pdg.native.PD_MIXED)
    m.step(15)
    u = ctx.state()[0]
    if np.abs(u).max() > 0:
        assert normwise(m.state()[0], u) < 1e-6
    # the host-buffer step (slabbed import; most slabs are empty at these sizes) agrees bit for bit
    h = p.context()
    bufs = [pdg.native.PinnedArray((n, 2)) for _ in range(3)]
    hu, hv, hf = (b.array for b in bufs)
    for b in (hu, hv, hf):
        b[:] = 0.0
    for k in (1, 2, 1):
        h.step_host(k, hu, hv, hf)
    ref = p.context()
    ref.step(4)
    for got, want in zip((hu, hv, hf), ref.state()):
        assert np.array_equal(got, want)
    for b in bufs:
        b.free()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_batch_with_degenerate_members(pdg, precision, mode):
    """A batch whose members include an empty problem, single particles and partial
    chunks next to a cracked plate: every member equals its solo run in every launch mode."""
    base = pdg.plates.make_plate(20, seed=6, crack="centre-half")
    base.material.s_c = 2e-4
    plates = [_subset(base, np.arange(n)) for n in (1, 2, 33, 257)] + [base]
    steps = 12
    solo = []
    for p in plates:
        c = p.context(precision=precision)
        c.step(steps)
        solo.append((*c.state(), c.bond_mask()))
        c.close()
    b = pdg.Batch(precision=precision)
    b.set_config(persistent=mode)
    empty = pdg.native.Context(pdg.default_params(precision=precision))
    empty.set_particles(np.zeros((0, 2)), np.zeros(0))
    empty.build_families(1.0)
    b.add(empty)
    ctxs = [p.context(precision=precision) for p in plates]
    for c in ctxs:
        b.add(c)
    b.step(5)
    b.step(steps - 5)
    b.synchronize()
    for c, ref in zip(ctxs, solo):
        for g, r in zip((*c.state(), c.bond_mask()), ref):
            assert np.array_equal(g, r)
    assert empty.state()[0].shape == (0, 2)
    b.close()


def test_ragged_families_with_holes(pdg, po):
    """Two circular holes and a slot: families from 0 to 28 bonds, particles
    with no neighbours (singular), SELL chunks of very different widths."""
    p = pdg.plates.make_plate(64, seed=8, crack="centre-half")
    p.material.s_c = 3e-4
    c = p.x / p.dx
    hole = (((c[:, 0] - 10) ** 2 + (c[:, 1] - 8) ** 2) < 81) | (((c[:, 0] + 12) ** 2 + (c[:, 1] + 5) ** 2) < 20)
    slot = (np.abs(c[:, 1] - 20) < 1.2) & (c[:, 0] > -5)
    lone = np.zeros_like(hole)
    for cx, cy in ((10, 8), (-12, -5)):  # one isolated particle left at each hole's centre
        lone[np.argmin((c[:, 0] - cx) ** 2 + (c[:, 1] - cy) ** 2)] = True
    q = _subset(p, np.nonzero(~(hole | slot) | lone)[0])
    ctx = q.context()
    sim = plate_oracle(po, q)
    fam = np.diff(sim.row_ptr)
    assert fam.min() == 0 and fam.max() >= 26
    for chunk in (5, 20):
        ctx.step(chunk)
        sim.step(chunk)
        _assert_same(ctx, sim)
    m = q.context(precision=pdg.native.PD_MIXED)
    m.step(25)
    assert normwise(m.state()[0], ctx.state()[0]) < 1e-6
    assert np.array_equal(m.bond_mask(), ctx.bond_mask())


def test_largest_families(pdg, po):
    """Horizon 5.9 dx: ~109 bonds per particle, close to PD_MAX_FAMILY = 128."""
    p = pdg.plates.make_plate(40, seed=2, horizon=5.9, crack="centre-half")
    ctx = p.context(s_c=0.0)
    sim = plate_oracle(po, p, s_c=0.0)
    assert 100 <= np.diff(sim.row_ptr).max() <= 128
    ctx.step(6)
    sim.step(6)
    _assert_same(ctx, sim)
    m = p.context(precision=pdg.native.PD_MIXED, s_c=0.0)
    m.step(6)
    assert normwise(m.state()[0], ctx.state()[0]) < 1e-6


def test_family_overflow_is_an_error(pdg):
    p = pdg.plates.make_plate(30, seed=2, horizon=7.0)  # ~154 bonds > PD_MAX_FAMILY
    with pytest.raises(pdg.PdError):
        p.context()


def test_bad_particles_rejected(pdg):
    ctx = pdg.native.Context(pdg.default_params())
    with pytest.raises(pdg.PdError):
        ctx.set_particles(np.array([[0.0, 0.0], [np.nan, 1.0]]), np.ones(2))
    with pytest.raises(pdg.PdError):
        ctx.set_particles(np.array([[0.0, 0.0], [1.0, 1.0]]), np.array([1.0, 0.0]))
    with pytest.raises(pdg.PdError):
        ctx.step(1)  # no families yet


def test_probes_report_plausible_rates(pdg):
    """The measured denominators the bench reports: the FP64 / FP32 FMA rates
    (FP64 well below FP32 on this part) and the copy-engine link rates
    (positive, below any CPU-GPU link's nominal peak), and bad arguments are
    refused."""
    fp64, fp32 = pdg.native.probe_fma_rates(0)
    assert 0 < fp64 < fp32
    h2d, d2h, both = pdg.native.probe_link_rates(16 << 20, 0)
    for r in (h2d, d2h, both):
        assert 1.0 < r < 2000.0
    with pytest.raises(pdg.PdError):
        pdg.native.probe_link_rates(8, 0)
