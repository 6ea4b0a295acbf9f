"""Host logic: plate generator, family rules, and size-independent properties
of the oracle's step (the properties the GPU tests check at full size)."""
import numpy as np

from conftest import plate_oracle


def test_plate_generator_deterministic(pdg):
    a = pdg.plates.make_plate(50, seed=7, crack="centre-half")
    b = pdg.plates.make_plate(50, seed=7, crack="centre-half")
    c = pdg.plates.make_plate(50, seed=8, crack="centre-half")
    assert np.array_equal(a.x, b.x) and not np.array_equal(a.x, c.x)
    assert np.abs(a.x[:, 0] - np.round(a.x[:, 0] / a.dx) * a.dx).max() <= 0.01 * a.dx * (1 + 1e-9)
    assert (a.group_of == 1).sum() == 150 and (a.group_of == 2).sum() == 150


def test_dt_is_0p8_cfl(pdg):
    p = pdg.plates.config_plate_100()
    assert abs(p.dt - 0.8 * 1e-3 / np.sqrt(72e9 / 2440.0)) < 1e-20


def test_families_28_stencil_and_crack(po, pdg):
    p = pdg.plates.config_plate_100(seed=1)
    rp0, _ = po.build_families(p.x, p.cutoff)
    rp, col = po.build_families(p.x, p.cutoff, p.cracks)
    deg0 = np.diff(rp0).reshape(100, 100)
    assert deg0[3:97, 3:97].min() == 28 and deg0.max() == 28
    assert rp0[-1] == 272836  # 100 x 100 directed bond count of the 28-offset stencil
    removed = rp0[-1] - rp[-1]
    assert removed > 0
    # a kept bond never crosses the crack segment; every dropped bond does
    yc, xa, xb = p.cracks[0, 1], p.cracks[0, 0], p.cracks[0, 2]

    def crossing(i, j):
        yi, yj = p.x[i, 1] - yc, p.x[j, 1] - yc
        straddle = yi * yj < 0
        t = np.where(straddle, yi / np.where(straddle, yi - yj, 1.0), 0.0)
        xint = p.x[i, 0] + t * (p.x[j, 0] - p.x[i, 0])
        return straddle & (xint > xa) & (xint < xb)

    i = np.repeat(np.arange(p.n), np.diff(rp))
    assert not crossing(i, col).any()
    i0 = np.repeat(np.arange(p.n), np.diff(rp0))
    _, col0 = po.build_families(p.x, p.cutoff)
    assert crossing(i0, col0).sum() == removed


def test_scale_plate_bond_count(pdg, po):
    # the 1000 x 1000 count quoted for the workload, via the 200 x 200 cut formula
    p = pdg.plates.make_plate(200, seed=0)
    rp, _ = po.build_families(p.x, p.cutoff)
    # 28-offset stencil on an n x n grid: sum over offsets (n-|dx|)(n-|dy|)
    offs = [(a, b) for a in range(-3, 4) for b in range(-3, 4) if 0 < a * a + b * b <= 9]
    assert len(offs) == 28
    count = lambda n: sum((n - abs(a)) * (n - abs(b)) for a, b in offs)
    assert rp[-1] == count(200)
    assert count(1000) == 27928036


def test_oracle_momentum_and_mask_symmetry(po, pdg):
    p = pdg.plates.make_plate(40, seed=2, crack="centre-half")
    sim = plate_oracle(po, p, s_c=2e-4)
    sim.step(40)
    # internal forces cancel: sum_i V_i f_i = 0 (gather form is antisymmetric per bond)
    tot = (p.vol[:, None] * sim.f).sum(0)
    scale = (p.vol[:, None] * np.abs(sim.f)).sum(0).max()
    assert np.abs(tot).max() < 1e-12 * scale
    # bond (i,j) and (j,i) break together
    i = np.repeat(np.arange(p.n), np.diff(sim.row_ptr))
    j = sim.col
    key = dict(zip(zip(i.tolist(), j.tolist()), sim.mask.tolist()))
    assert all(key[(b, a)] == m for (a, b), m in key.items())
    assert sim.mask.min() == 0
    # damage = broken / family size
    broken = np.bincount(i, weights=(sim.mask == 0), minlength=p.n)
    assert np.array_equal(sim.damage, broken / np.diff(sim.row_ptr))


def test_oracle_threads_do_not_change_results(po, pdg):
    p = pdg.plates.make_plate(36, seed=4, crack="centre-half")
    a = plate_oracle(po, p, s_c=2e-4)
    a.nthreads = 1
    a._pb.nthreads = 1
    b = plate_oracle(po, p, s_c=2e-4)
    b.nthreads = 3
    b._pb.nthreads = 3
    a.step(25)
    b.step(25)
    assert np.array_equal(a.u, b.u) and np.array_equal(a.f, b.f) and np.array_equal(a.mask, b.mask)
