"""Particles of unequal volume.

Every generated plate and the reference's mesh give all particles the same
volume, which lets the mixed form's single-plate pass A leave the V_j gathers
out (the host checks that every (float)(V_i / V_mean) is exactly 1).  Here each
particle's volume carries a seeded factor in [0.75, 1.25], as a mesh of mixed
cell sizes would, so the mixed form runs its general pass A, and the FP64 form
weights every bond by an individual V_j.  Bars: the FP64 form bit-identical to
the oracle; the mixed form within 1e-6 of FP64 with the same broken-bond mask;
the batched mixed step bit-identical to the solo one.
"""
import dataclasses

import numpy as np
import pytest

from conftest import normwise, plate_oracle

pytestmark = pytest.mark.gpu


def _graded(pdg, side, seed, s_c=2e-4):
    mat = pdg.plates.Material()
    mat.s_c = s_c  # bonds break within the runs
    p = pdg.plates.make_plate(side, seed=seed, crack="centre-half", material=mat)
    f = np.random.default_rng(seed + 100).uniform(0.75, 1.25, p.n)
    q = dataclasses.replace(p, vol=np.ascontiguousarray(p.vol * f))
    assert np.unique(q.vol).size > p.n // 2
    return q


def test_gpu_fp64_graded_volumes_bit_exact(pdg, po):
    p = _graded(pdg, 48, seed=4)
    ctx = p.context()
    sim = plate_oracle(po, p)
    for chunk in (10, 70):
        ctx.step(chunk)
        sim.step(chunk)
        u, v, f = ctx.state()
        assert np.array_equal(u, sim.u) and np.array_equal(v, sim.v) and np.array_equal(f, sim.f)
        assert np.array_equal(ctx.bond_mask(), sim.mask)
        assert np.array_equal(ctx.damage(), sim.damage)
    assert sim.mask.min() == 0, "the case is meant to break bonds"


def test_mixed_graded_volumes_against_fp64(pdg):
    p = _graded(pdg, 120, seed=6)
    a = p.context(precision=pdg.native.PD_FP64)
    b = p.context(precision=pdg.native.PD_MIXED)
    for target, done in ((100, 0), (300, 100)):
        a.step(target - done)
        b.step(target - done)
        ua, ub = a.state()[0], b.state()[0]
        err = normwise(ub, ua)
        mm = int((a.bond_mask() != b.bond_mask()).sum())
        print(f"graded volumes, 120x120, step {target}: u_max_rel {err:.3e}, mask mismatches {mm}")
        assert err < 1e-6
        assert mm == 0
    assert int((a.bond_mask() == 0).sum()) > 0, "the run is meant to break bonds"


def test_mixed_graded_volumes_batch_equals_solo(pdg):
    plates = [_graded(pdg, side, seed) for side, seed in ((40, 1), (57, 2), (33, 3))]
    steps = 40
    solo = []
    for p in plates:
        c = p.context(precision=pdg.native.PD_MIXED)
        c.step(steps)
        solo.append((*c.state(), c.bond_mask(), c.damage()))
        c.close()
    b = pdg.Batch(precision=pdg.native.PD_MIXED)
    ctxs = [p.context(precision=pdg.native.PD_MIXED) for p in plates]
    for c in ctxs:
        b.add(c)
    b.step(steps)
    b.synchronize()
    broke = 0
    for c, ref in zip(ctxs, solo):
        for g, r in zip((*c.state(), c.bond_mask(), c.damage()), ref):
            assert np.array_equal(g, r)
        broke += int((ref[3] == 0).sum())
    assert broke > 0
