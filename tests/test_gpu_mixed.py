"""Mixed form (PD_MIXED) vs the FP64 form.

The FP64 GPU path is bit-identical to the oracle (test_gpu_fp64_parity.py),
so it serves as the FP64 oracle at sizes the CPU restatement would take long
on.  Bars: <= 1e-6 normwise relative displacement error and an
identical damage mask; the velocity error and mask mismatches are reported.
"""
import numpy as np
import pytest

from conftest import normwise

pytestmark = pytest.mark.gpu

DISP_TOL = 1e-6


def _pair(pdg, plate):
    a = plate.context(precision=pdg.native.PD_FP64)
    b = plate.context(precision=pdg.native.PD_MIXED)
    return a, b


def _errors(a, b):
    ua, va, fa = a.state()
    ub, vb, fb = b.state()
    ma, mb = a.bond_mask(), b.bond_mask()
    rms = float(np.sqrt(((ub - ua) ** 2).mean()) / np.sqrt((ua ** 2).mean()))
    return {"u_max": normwise(ub, ua), "u_rms": rms, "v_max": normwise(vb, va), "f_max": normwise(fb, fa),
            "mask_mismatch": int((ma != mb).sum()), "broken": int((ma == 0).sum())}


def test_mixed_config1_100_steps(pdg):
    p = pdg.plates.config_plate_100(seed=0)
    a, b = _pair(pdg, p)
    a.step(100)
    b.step(100)
    e = _errors(a, b)
    print("mixed vs fp64, 100x100, 100 steps:", e)
    assert e["u_max"] < DISP_TOL
    assert e["mask_mismatch"] == 0


@pytest.mark.parametrize("nx,ny", [(160, 80), (70, 140)])
def test_mixed_rectangular_plates(pdg, nx, ny):
    """2:1 plates (the serving workload's other shape; tiles cut both edges) with an
    angled pre-crack and breaking: the mixed form stays within the bar of FP64 with the
    same broken-bond mask."""
    mat = pdg.plates.Material()
    mat.s_c = 2e-4  # bonds break within the run
    p = pdg.plates.make_plate(nx, ny, seed=5, crack=(0.0, 0.0, 0.4 * min(nx, ny) * 1e-3, 0.35), material=mat,
                              v_load=1.5)
    a, b = _pair(pdg, p)
    a.step(300)
    b.step(300)
    e = _errors(a, b)
    print(f"mixed vs fp64, {nx}x{ny}, 300 steps:", e)
    assert e["u_max"] < DISP_TOL
    assert e["mask_mismatch"] == 0
    assert int((a.bond_mask() == 0).sum()) > 0  # the run did break bonds


def test_mixed_200_cut_to_1000_steps(pdg):
    """The 200 x 200 cut of the scale plate (same generator), errors at steps 100/500/1000."""
    p = pdg.plates.config_plate_scale(side=200, seed=0)
    a, b = _pair(pdg, p)
    done = 0
    report = {}
    for target in (100, 500, 1000):
        a.step(target - done)
        b.step(target - done)
        done = target
        report[target] = _errors(a, b)
    print("mixed vs fp64, 200x200:", report)
    for t, e in report.items():
        assert e["u_max"] < DISP_TOL, (t, e)
    assert report[1000]["broken"] > 0, "the run is meant to break bonds"
    for t, e in report.items():
        assert e["mask_mismatch"] == 0, (t, e)  # an identical damage mask


def test_mixed_400_cut_identical_mask_at_100_500_1000(pdg):
    """A 400 x 400 cut of the 1M-particle workload (160,000 particles, ~4.4M
    bonds, its own seeded crack), mixed against FP64 at steps 100/500/1000:
    displacements within the 1e-6 bar and the same broken-bond mask."""
    p = pdg.plates.config_plate_scale(side=400, seed=0)
    a, b = _pair(pdg, p)
    done = 0
    report = {}
    for target in (100, 500, 1000):
        a.step(target - done)
        b.step(target - done)
        done = target
        report[target] = _errors(a, b)
    print("mixed vs fp64, 400x400:", report)
    assert report[1000]["broken"] > 1000, "the run is meant to break bonds"
    for t, e in report.items():
        assert e["u_max"] < DISP_TOL, (t, e)
        assert e["mask_mismatch"] == 0, (t, e)


def test_mixed_state_roundtrip_and_determinism(pdg):
    p = pdg.plates.make_plate(64, seed=3, crack="centre-half")
    b = p.context(precision=pdg.native.PD_MIXED)
    b.step(20)
    u, v, f = b.state()
    b.set_state(u=u, v=v, f=f)
    u2, v2, f2 = b.state()
    assert normwise(u2, u) < 1e-13 and normwise(v2, v) < 1e-13 and normwise(f2, f) < 1e-7
    c = p.context(precision=pdg.native.PD_MIXED)
    c.step(20)
    for x, y in zip((u, v, f), c.state()):
        assert np.array_equal(x, y)


def test_mixed_rejects_dropin_call(pdg):
    p = pdg.plates.make_plate(16, seed=1)
    b = p.context(precision=pdg.native.PD_MIXED)
    u = np.zeros((p.n, 2))
    with pytest.raises(pdg.PdError):
        b.compute_velocity(u, np.zeros((p.n, 2)), np.zeros((p.n, 2)))


def test_mixed_shuffled_numbering_matches(pdg):
    """Particles numbered in a random order.  The mixed form lays its chunks
    and visiting blocks out by position and walks every family in spatial
    order, so after undoing the permutation the result is bit-identical to
    the row-major run, and agrees with the FP64 form on the shuffled plate
    within the mixed-form bar."""
    import dataclasses
    p = pdg.plates.make_plate(120, seed=5, crack="centre-half")
    perm = np.random.default_rng(7).permutation(p.n)
    q = dataclasses.replace(p, x=np.ascontiguousarray(p.x[perm]), vol=np.ascontiguousarray(p.vol[perm]),
                            group_of=np.ascontiguousarray(p.group_of[perm]))
    a = q.context(precision=pdg.native.PD_FP64)
    b = q.context(precision=pdg.native.PD_MIXED)
    r = p.context(precision=pdg.native.PD_MIXED)
    assert b.counters()["unstaged_blocks"] == 0 and r.counters()["unstaged_blocks"] == 0
    for c in (a, b, r):
        c.step(200)
    e = _errors(a, b)
    print("shuffled numbering, mixed vs fp64:", e)
    assert e["u_max"] < DISP_TOL
    assert e["broken"] > 0 and e["mask_mismatch"] == 0
    for got, want in zip(b.state(), r.state()):
        assert np.array_equal(got, want[perm])
    assert np.array_equal(b.damage(), r.damage()[perm])


def test_mixed_on_the_reference_mesh(pdg, hassa):
    """The reference's own mesh (its Hassa test mesh: 4,064 particles,
    irregular spacing) under the reference main's loading: every visiting
    block of the spatial layout stages its halo, and the mixed form agrees
    with the FP64 form within the mixed-form bar after 100 steps."""
    n = hassa["x"].shape[0]
    dx, hor, E, nu, rho, dt = hassa["params"]
    g = np.zeros(n, np.uint8)
    g[hassa["top"]] = 1
    g[hassa["bottom"]] = 2
    ctxs = []
    for prec in (pdg.native.PD_FP64, pdg.native.PD_MIXED):
        c = pdg.native.Context(pdg.default_params(E=E, nu=nu, rho=rho, dt=dt, s_c=0.0, precision=prec))
        c.set_particles(hassa["x"], hassa["vol"])
        c.build_families(1.01 * dx * hor)
        c.set_bc([pdg.native.PD_BC_VELOCITY, pdg.native.PD_BC_FIXED], [[0.0, 5.0], [0.0, 0.0]], g)
        ctxs.append(c)
    a, b = ctxs
    assert np.array_equal(a.families()[1], b.families()[1])
    assert b.counters()["unstaged_blocks"] == 0
    for c in ctxs:
        c.step(100)
    e = _errors(a, b)
    print("reference mesh, mixed vs fp64:", e)
    assert e["u_max"] < DISP_TOL


def test_mixed_dense_cluster_unstaged_blocks(pdg):
    """A 120 x 120 plate with scrambled numbering and two lone particles 10 m
    apart: the layout's cells follow the bounding box, so each holds thousands
    of plate particles, its tile (more than 2,048 particles) is ordered on the
    host, and a block's 256 particles are scattered over a cell, reaching more
    particles than a block can stage.  Those blocks gather neighbour data from
    HBM; the result agrees with the FP64 form within the mixed-form bar."""
    import dataclasses
    p = pdg.plates.make_plate(120, seed=5, crack="centre-half")
    perm = np.random.default_rng(11).permutation(p.n)
    far = np.array([[-5.0, -5.0], [5.0, 5.0]])
    q = dataclasses.replace(p, x=np.ascontiguousarray(np.vstack([p.x[perm], far])),
                            vol=np.ascontiguousarray(np.concatenate([p.vol[perm], p.vol[:2]])),
                            group_of=np.ascontiguousarray(np.concatenate([p.group_of[perm],
                                                                          np.zeros(2, p.group_of.dtype)])))
    a = q.context(precision=pdg.native.PD_FP64)
    b = q.context(precision=pdg.native.PD_MIXED)
    assert b.counters()["unstaged_blocks"] > 0
    assert a.counters()["unstaged_blocks"] == 0
    for c in (a, b):
        c.step(200)
    e = _errors(a, b)
    print("dense cluster, mixed vs fp64:", e, "unstaged blocks:", b.counters()["unstaged_blocks"])
    assert e["u_max"] < DISP_TOL
    assert e["broken"] > 0 and e["mask_mismatch"] == 0


@pytest.mark.parametrize("precision", [0, 1])
def test_checkpoint_restore_continues_bit_for_bit(pdg, precision):
    """Save after 30 steps, run 25 more; a fresh context of the same plate
    restored from the blob and run 25 steps ends in the identical state."""
    p = pdg.plates.make_plate(72, seed=11, crack="centre-half")
    p.material.s_c = 2e-4  # bonds break before and after the checkpoint
    a = p.context(precision=precision)
    a.step(30)
    blob = a.checkpoint()
    broken_at_save = a.counters()["bonds_broken"]
    a.step(25)
    b = p.context(precision=precision)
    b.restore(blob)
    assert b.counters()["steps"] == 30 and b.counters()["bonds_broken"] == broken_at_save
    b.step(25)
    for x, y in zip((*a.state(), a.bond_mask(), a.damage()), (*b.state(), b.bond_mask(), b.damage())):
        assert np.array_equal(x, y)
    ca, cb = a.counters(), b.counters()
    assert ca == cb and ca["bonds_broken"] > broken_at_save > 0


def test_checkpoint_rejects_other_problems(pdg):
    p = pdg.plates.make_plate(40, seed=1)
    q = pdg.plates.make_plate(40, seed=2)  # same size, other jitter
    a = p.context(precision=pdg.native.PD_MIXED)
    a.step(3)
    blob = a.checkpoint()
    with pytest.raises(pdg.PdError):
        q.context(precision=pdg.native.PD_MIXED).restore(blob)
    with pytest.raises(pdg.PdError):
        p.context(precision=pdg.native.PD_FP64).restore(blob)
    with pytest.raises(pdg.PdError):
        p.context(precision=pdg.native.PD_MIXED).restore(blob[:-8])
    c = p.context(precision=pdg.native.PD_MIXED)
    c.restore(blob)  # the matching context accepts it
    assert c.counters()["steps"] == 3


@pytest.mark.parametrize("shuffle", [False, True])
def test_mixed_step_host_equals_staged_copies(pdg, shuffle):
    """pd_step_host on a mixed context (import + drift of each slab read over
    the CPU-GPU link, passes in a wavefront of slabs, the last pass B writing
    the FP64 state to the host buffers) is pd_set_state + pd_step +
    pd_get_state, bit for bit, call after call while bonds break -- with the
    plate numbered row-major (slabs reach their neighbours only) and randomly
    (every slab reaches every other one)."""
    import dataclasses
    p = pdg.plates.make_plate(240, seed=4, crack="centre-half")
    p.material.s_c = 2e-4
    if shuffle:
        perm = np.random.default_rng(3).permutation(p.n)
        p = dataclasses.replace(p, x=np.ascontiguousarray(p.x[perm]), vol=np.ascontiguousarray(p.vol[perm]),
                                group_of=np.ascontiguousarray(p.group_of[perm]))
    a = p.context(precision=pdg.native.PD_MIXED)
    b = p.context(precision=pdg.native.PD_MIXED)
    a.step(7)
    b.step(7)
    u, v, f = a.state()
    bufs = [pdg.native.PinnedArray((p.n, 2)) for _ in range(6)]
    hu, hv, hf, ou, ov, of = (x.array for x in bufs)
    hu[:], hv[:], hf[:] = u, v, f
    broke = 0
    for call, nsteps in enumerate((1, 1, 3, 1, 2, 1)):
        a.set_state(u=hu, v=hv, f=hf)
        a.step(nsteps)
        ua, va, fa = a.state()
        if call % 2:  # separate output buffers, then in place
            b.step_host(nsteps, hu, hv, hf, ou, ov, of)
            hu[:], hv[:], hf[:] = ou, ov, of
        else:
            b.step_host(nsteps, hu, hv, hf)
        assert np.array_equal(ua, hu) and np.array_equal(va, hv) and np.array_equal(fa, hf), (call, nsteps)
        assert np.array_equal(a.bond_mask(), b.bond_mask())
        broke = int((b.bond_mask() == 0).sum())
    assert broke > 0
    for x in bufs:
        x.free()


@pytest.mark.parametrize("case", ["tiny", "one_row_of_tiles", "dense_cluster"])
def test_mixed_step_host_edge_layouts(pdg, case):
    """pd_step_host on layouts that stress the slab plan: a plate of one visiting
    block (most slabs empty), a plate one tile high (every slab a run of
    neighbouring tiles), and a scrambled plate whose blocks are not staged
    (they gather from HBM; their bonds reach across every slab) -- each equal,
    bit for bit, to pd_set_state + pd_step + pd_get_state, one step and three."""
    import dataclasses
    if case == "tiny":
        p = pdg.plates.make_plate(9, seed=3)
    elif case == "one_row_of_tiles":
        p = pdg.plates.make_plate(512, 8, seed=3, bc_rows=2)
    else:
        p = pdg.plates.make_plate(120, seed=5, crack="centre-half")
        perm = np.random.default_rng(11).permutation(p.n)
        far = np.array([[-5.0, -5.0], [5.0, 5.0]])
        p = dataclasses.replace(p, x=np.ascontiguousarray(np.vstack([p.x[perm], far])),
                                vol=np.ascontiguousarray(np.concatenate([p.vol[perm], p.vol[:2]])),
                                group_of=np.ascontiguousarray(np.concatenate([p.group_of[perm],
                                                                              np.zeros(2, p.group_of.dtype)])))
    a = p.context(precision=pdg.native.PD_MIXED)
    b = p.context(precision=pdg.native.PD_MIXED)
    if case == "dense_cluster":
        assert b.counters()["unstaged_blocks"] > 0
    a.step(5)
    b.step(5)
    bufs = [pdg.native.PinnedArray((p.n, 2)) for _ in range(3)]
    hu, hv, hf = (x.array for x in bufs)
    hu[:], hv[:], hf[:] = a.state()
    for nsteps in (1, 3, 1):
        a.set_state(u=hu, v=hv, f=hf)
        a.step(nsteps)
        ua, va, fa = a.state()
        b.step_host(nsteps, hu, hv, hf)
        assert np.array_equal(ua, hu) and np.array_equal(va, hv) and np.array_equal(fa, hf), (case, nsteps)
        assert np.array_equal(a.bond_mask(), b.bond_mask())
    for x in bufs:
        x.free()
