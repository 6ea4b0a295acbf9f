"""FP64 CUDA path (through the C ABI) vs the oracle and the reference fixtures.

The FP64 kernels perform the oracle's IEEE operations in the oracle's order
(--fmad=false + the same explicit fma() calls), so the bar here is bit
equality for displacements, velocities, forces, the bond mask and damage;
against the reference's own outputs the bar is 1e-10
(normwise) on velocities/displacements, see test_oracle_golden.py for the
reference's long-double floor on the Hassa mesh.
"""
import numpy as np
import pytest

from conftest import hassa_oracle, normwise, plate_oracle
from test_oracle_golden import F_TOL, V_TOL, u_tol

pytestmark = pytest.mark.gpu


def _hassa_ctx(pdg, h):
    n = h["x"].shape[0]
    dx, hor, E, nu, rho, dt = h["params"]
    ctx = pdg.native.Context(pdg.default_params(E=E, nu=nu, rho=rho, dt=dt, s_c=0.0))
    ctx.set_particles(h["x"], h["vol"])
    ctx.build_families(1.01 * dx * hor)
    g = np.zeros(n, np.uint8)
    g[h["top"]] = 1
    g[h["bottom"]] = 2
    ctx.set_bc([pdg.native.PD_BC_VELOCITY, pdg.native.PD_BC_FIXED], [[0.0, 5.0], [0.0, 0.0]], g)
    return ctx


def _assert_same(ctx, sim):
    u, v, f = ctx.state()
    assert np.array_equal(u, sim.u), f"u differs: {np.abs(u - sim.u).max()}"
    assert np.array_equal(v, sim.v), f"v differs: {np.abs(v - sim.v).max()}"
    assert np.array_equal(f, sim.f), f"f differs: {np.abs(f - sim.f).max()}"
    assert np.array_equal(ctx.bond_mask(), sim.mask)
    assert np.array_equal(ctx.damage(), sim.damage)


def test_gpu_families_hassa_match_reference(pdg, hassa):
    ctx = _hassa_ctx(pdg, hassa)
    rp, col = ctx.families()
    assert np.array_equal(rp, hassa["row_ptr"]) and np.array_equal(col, hassa["col"])


def test_gpu_families_plate_with_crack_match_oracle(pdg, po):
    p = pdg.plates.config_plate_100(seed=5)
    ctx = p.context()
    rp, col = ctx.families()
    orp, ocol = po.build_families(p.x, p.cutoff, p.cracks)
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    assert int(np.diff(rp).max()) == 28


def test_gpu_hassa_matches_reference_fixture(pdg, po, hassa):
    ctx = _hassa_ctx(pdg, hassa)
    ctx.step(1)
    u, v, f = ctx.state()
    assert normwise(v, hassa["c_v1"]) < V_TOL
    assert normwise(u, hassa["c_u1"]) < u_tol(hassa["x"], hassa["c_u1"])
    assert normwise(f, hassa["c_f1"]) < F_TOL
    ctx.step(2)
    u, v, f = ctx.state()
    assert normwise(v, hassa["c_v3"]) < V_TOL
    assert normwise(u, hassa["c_u3"]) < u_tol(hassa["x"], hassa["c_u3"])
    assert normwise(f, hassa["c_f3"]) < F_TOL
    sim = hassa_oracle(po, hassa)
    sim.step(3)
    _assert_same(ctx, sim)


def test_gpu_plate30_matches_reference_fixture(pdg, plate30_ref):
    p = pdg.plates.make_plate(30, seed=3, crack="centre-half")
    ctx = p.context(s_c=0.0, k_hg=0.0)  # the reference's model (no zero-energy-mode penalty)
    rp, col = ctx.families()
    assert np.array_equal(rp, plate30_ref["row_ptr"]) and np.array_equal(col, plate30_ref["col"])
    ctx.step(1)
    u, v, f = ctx.state()
    assert normwise(u, plate30_ref["u1"]) < V_TOL and normwise(v, plate30_ref["v1"]) < V_TOL
    assert normwise(f, plate30_ref["f1"]) < F_TOL
    ctx.step(3)
    u, v, f = ctx.state()
    assert normwise(u, plate30_ref["u4"]) < V_TOL and normwise(v, plate30_ref["v4"]) < V_TOL
    assert normwise(f, plate30_ref["f4"]) < F_TOL


@pytest.mark.parametrize("side,seed,s_c,steps", [(48, 1, 5e-4, 60), (64, 2, 2e-4, 40), (33, 4, 0.0, 10)])
def test_gpu_fp64_bit_exact_vs_oracle(pdg, po, side, seed, s_c, steps):
    p = pdg.plates.make_plate(side, seed=seed, crack="centre-half")
    ctx = p.context(s_c=s_c)
    sim = plate_oracle(po, p, s_c=s_c)
    done = 0
    for chunk in (1, 2, steps - 3):  # graph per distinct step count, state carried across calls
        ctx.step(chunk)
        sim.step(chunk)
        done += chunk
        _assert_same(ctx, sim)
    if s_c > 0:
        assert sim.mask.min() == 0, "the case is meant to break bonds"
        assert ctx.counters()["bonds_broken"] == int((sim.mask == 0).sum())


@pytest.mark.parametrize("nx,ny", [(80, 40), (36, 72)])
def test_gpu_fp64_rectangular_angled_crack_bit_exact(pdg, po, nx, ny):
    """2:1 plates with an angled pre-crack off the centre (the serving workload's shapes)."""
    mat = pdg.plates.Material()
    mat.s_c = 2e-4
    p = pdg.plates.make_plate(nx, ny, seed=9, crack=(0.004, -0.002, 0.4 * min(nx, ny) * 1e-3, -0.4), material=mat,
                              v_load=1.5)
    ctx = p.context()
    sim = plate_oracle(po, p)
    for chunk in (5, 45):
        ctx.step(chunk)
        sim.step(chunk)
        _assert_same(ctx, sim)
    assert sim.mask.min() == 0, "the case is meant to break bonds"


def test_gpu_config1_plate_100_steps_bit_exact(pdg, po):
    """The CPU-runnable plate: 100x100, centred half-width crack, s_c = 5e-4, 100 steps."""
    p = pdg.plates.config_plate_100(seed=0)
    ctx = p.context()
    sim = plate_oracle(po, p)
    ctx.step(100)
    sim.step(100)
    _assert_same(ctx, sim)


def test_gpu_compute_velocity_dropin_matches_oracle(pdg, po):
    """pd_compute_velocity (compute_velocity_GPU_host contract) after a host drift."""
    p = pdg.plates.make_plate(40, seed=9, crack="centre-half")
    ctx = p.context(s_c=0.0)
    sim = plate_oracle(po, p, s_c=0.0)
    sim.step(3)
    # host-side drift of the next step, as the reference host loop does
    u, v, f = sim.u.copy(), sim.v.copy(), sim.f.copy()
    top, bot = p.group_of == 1, p.group_of == 2
    v[top] = p.group_val[0]
    v[bot] = p.group_val[1]
    a = f * (1.0 / p.material.rho)
    u = u + (v * p.dt + (0.5 * a) * (p.dt * p.dt))
    vel, acc = v.copy(), a.copy()
    ctx.set_state(u=u, v=v, f=f)
    netf = ctx.compute_velocity(u, vel, acc)
    sim.step(1)
    assert np.array_equal(netf, sim.f)
    assert np.array_equal(vel, sim.v)
    assert np.array_equal(acc, sim.f * (1.0 / p.material.rho))


def test_gpu_reset_and_determinism(pdg):
    p = pdg.plates.make_plate(80, seed=6, crack="centre-half")
    ctx = p.context(s_c=3e-4)
    ctx.step(30)
    a = ctx.state()
    m = ctx.bond_mask()
    ctx.reset()
    ctx.step(30)
    b = ctx.state()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert np.array_equal(m, ctx.bond_mask())


def test_gpu_set_families_from_host(pdg, po):
    p = pdg.plates.make_plate(24, seed=8, crack="centre-half")
    rp, col = po.build_families(p.x, p.cutoff, p.cracks)
    ctx = pdg.native.Context(p.params())
    ctx.set_particles(p.x, p.vol)
    ctx.set_families(rp, col)
    ctx.set_bc(p.group_kind, p.group_val, p.group_of)
    sim = plate_oracle(po, p, families=(rp, col))
    ctx.step(5)
    sim.step(5)
    _assert_same(ctx, sim)


def test_gpu_rejects_bad_families(pdg):
    p = pdg.plates.make_plate(8, seed=1)
    ctx = pdg.native.Context(p.params())
    ctx.set_particles(p.x, p.vol)
    rp = np.arange(p.n + 1, dtype=np.int64)
    col = np.full(p.n, p.n + 5, dtype=np.int32)  # out of range
    with pytest.raises(pdg.PdError) as e:
        ctx.set_families(rp, col)
    assert e.value.code == -1
    with pytest.raises(pdg.PdError):
        ctx.step(1)  # no families -> PD_ERR_ORDER


def test_gpu_singular_policy(pdg):
    """Two collinear bonds only: det(K) = 0; ZERO policy gives S = 0, ERROR policy fails the step."""
    x = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0]])
    vol = np.ones(3)
    for policy, expect_err in ((0, False), (1, True)):
        ctx = pdg.native.Context(pdg.default_params(E=1.0, nu=0.2, rho=1.0, dt=1e-3, singular_policy=policy))
        ctx.set_particles(x, vol)
        ctx.build_families(1.5)
        if expect_err:
            with pytest.raises(pdg.PdError) as e:
                ctx.step(1)
            assert e.value.code == -5
        else:
            ctx.step(2)
            u, v, f = ctx.state()
            assert np.all(f == 0.0) and ctx.counters()["singular_events"] == 3


def test_gpu_step_host_equals_staged_copies(pdg):
    """pd_step_host (the state copied in by slabs while the first pass runs,
    written back by the last kernel over the CPU-GPU link) is pd_set_state +
    pd_step + pd_get_state, bit for bit, call after call while bonds break."""
    p = pdg.plates.make_plate(90, seed=4, crack="centre-half")
    p.material.s_c = 2e-4
    a = p.context()
    b = p.context()
    a.step(7)
    b.step(7)
    u, v, f = a.state()
    bufs = [pdg.native.PinnedArray((p.n, 2)) for _ in range(3)]
    hu, hv, hf = (x.array for x in bufs)
    hu[:], hv[:], hf[:] = u, v, f
    for nsteps in (1, 1, 3, 1, 2, 1):
        a.set_state(u=hu, v=hv, f=hf)
        a.step(nsteps)
        ua, va, fa = a.state()
        b.step_host(nsteps, hu, hv, hf)
        assert np.array_equal(ua, hu) and np.array_equal(va, hv) and np.array_equal(fa, hf)
        assert np.array_equal(a.bond_mask(), b.bond_mask())
    with pytest.raises(pdg.PdError):  # pageable numpy memory is refused
        b.step_host(1, u.copy(), v.copy(), f.copy())
    for x in bufs:
        x.free()


@pytest.mark.parametrize("case", ["one_chunk", "shuffled"])
def test_gpu_step_host_edge_layouts(pdg, case):
    """pd_step_host where the slab plan degenerates: 20 particles (one chunk, all
    but the first slab empty) and a randomly numbered plate (every slab's bonds
    reach every other slab, so each pass A waits for the whole import and each
    pass B for every pass A) -- bit for bit pd_set_state + pd_step + pd_get_state."""
    import dataclasses
    if case == "one_chunk":
        p = pdg.plates.make_plate(5, 4, seed=2, bc_rows=1)
    else:
        p = pdg.plates.make_plate(70, seed=4, crack="centre-half")
        perm = np.random.default_rng(7).permutation(p.n)
        p = dataclasses.replace(p, x=np.ascontiguousarray(p.x[perm]), vol=np.ascontiguousarray(p.vol[perm]),
                                group_of=np.ascontiguousarray(p.group_of[perm]))
    p.material.s_c = 2e-4
    a = p.context()
    b = p.context()
    a.step(4)
    b.step(4)
    bufs = [pdg.native.PinnedArray((p.n, 2)) for _ in range(3)]
    hu, hv, hf = (x.array for x in bufs)
    hu[:], hv[:], hf[:] = a.state()
    for nsteps in (1, 2, 1):
        a.set_state(u=hu, v=hv, f=hf)
        a.step(nsteps)
        ua, va, fa = a.state()
        b.step_host(nsteps, hu, hv, hf)
        assert np.array_equal(ua, hu) and np.array_equal(va, hv) and np.array_equal(fa, hf), (case, nsteps)
        assert np.array_equal(a.bond_mask(), b.bond_mask())
    for x in bufs:
        x.free()


@pytest.mark.parametrize("case", ["plate", "one_chunk", "shuffled"])
def test_gpu_compute_velocity_pinned_equals_staged(pdg, case):
    """pd_compute_velocity on page-locked buffers (pd_step_host's slab pipeline,
    each slab's pass B writing velocity, acce and the force back) against the
    same calls on pageable buffers (whole-array copies): bit for bit, velocity
    and acce in place, over repeated calls that break bonds, on a 300 x 300
    plate and on the layouts where the slab plan degenerates."""
    import dataclasses
    if case == "plate":
        p = pdg.plates.make_plate(300, seed=3, crack="centre-half")
    elif case == "one_chunk":
        p = pdg.plates.make_plate(5, 4, seed=2, bc_rows=1)
    else:
        p = pdg.plates.make_plate(70, seed=4, crack="centre-half")
        perm = np.random.default_rng(7).permutation(p.n)
        p = dataclasses.replace(p, x=np.ascontiguousarray(p.x[perm]), vol=np.ascontiguousarray(p.vol[perm]),
                                group_of=np.ascontiguousarray(p.group_of[perm]))
    p.material.s_c = 2e-4
    run = p.context()
    run.step(40)  # a strained state, so that the calls below break bonds
    u, v, f = run.state()
    run.close()
    acc = f / p.material.rho
    a = p.context()
    b = p.context()
    bufs = [pdg.native.PinnedArray((p.n, 2)) for _ in range(4)]
    hu, hv, ha, hf = (x.array for x in bufs)
    hu[:], hv[:], ha[:] = u, v, acc
    for _ in range(4):
        fa = a.compute_velocity(u, v, acc)  # pageable buffers: staged copies
        b.compute_velocity(hu, hv, ha, netf=hf)  # page-locked buffers: the slab pipeline
        assert np.array_equal(v, hv) and np.array_equal(acc, ha) and np.array_equal(fa, hf), case
        assert np.array_equal(a.bond_mask(), b.bond_mask()) and np.array_equal(a.damage(), b.damage())
        u = u + v * p.dt + 0.5 * acc * p.dt ** 2  # the reference host loop's drift, the same for both
        hu[:] = u
    if case != "one_chunk":
        assert int((a.bond_mask() == 0).sum()) > 0, "the calls are meant to break bonds"
    for x in bufs:
        x.free()


def test_gpu_scale_plate_200_cut_1000_steps_bit_exact(pdg, po):
    """The 1000 x 1000 workload's generator at 200 x 200 (same seed rule,
    seeded crack), 1000 steps with bond breaking: bit-exact damage mask,
    damage and state against the CPU restatement at steps 100, 500, 1000."""
    p = pdg.plates.config_plate_scale(side=200, seed=0)
    ctx = p.context()
    sim = plate_oracle(po, p)
    done = 0
    for target in (100, 500, 1000):
        ctx.step(target - done)
        sim.step(target - done)
        done = target
        _assert_same(ctx, sim)
    assert int((sim.mask == 0).sum()) > 0, "the crack is meant to run"


def test_gpu_concurrent_family_builds_match_sequential(pdg):
    """Contexts built on several threads at once, as the serving loop builds
    them, get the families of a build on its own: each family build carries
    its own crack segments."""
    import math
    from concurrent.futures import ThreadPoolExecutor
    plates = [pdg.plates.make_plate(150, seed=s, crack=(0.0, 0.004 * (s - 3), 0.02 + 0.015 * s,
                                                        math.radians(-30.0 + 12.0 * s))) for s in range(6)]
    want = []
    for p in plates:
        c = p.context()
        want.append(c.families())
        c.close()
    for _ in range(2):
        with ThreadPoolExecutor(max_workers=6) as ex:
            ctxs = list(ex.map(lambda p: p.context(), plates))
        for c, (rp, col) in zip(ctxs, want):
            grp, gcol = c.families()
            assert np.array_equal(grp, rp) and np.array_equal(gcol, col)
            c.close()
