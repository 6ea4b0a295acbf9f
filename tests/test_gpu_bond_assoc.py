"""Bond-associated mode (the reference's default n1 = n2 = 10 weights) on the GPU.

Against the reference's own full-precision output of that run (the run whose
6-digit velocities are the reference's shipped golden file,
output/velocity_step_0_after_seq_ref.txt -- tests/golden/manifest.json
pins it), and against the oracle's O(n^2) restatement over several steps.
exp/pow differ between CUDA and libm by rounding, so GPU vs oracle is
compared at 1e-12 normwise instead of bit for bit.
"""
import numpy as np
import pytest

from conftest import normwise
from test_oracle_golden import F_TOL, V_TOL, u_tol

pytestmark = pytest.mark.gpu


def _ctx(pdg, h, n1=10.0, n2=10.0):
    n = h["x"].shape[0]
    dx, hor, E, nu, rho, dt = h["params"]
    ctx = pdg.native.Context(pdg.default_params(E=E, nu=nu, rho=rho, dt=dt, s_c=0.0, n1=n1, n2=n2,
                                                weight_len=hor * dx))
    ctx.set_particles(h["x"], h["vol"])
    ctx.build_families(1.01 * dx * hor)
    g = np.zeros(n, np.uint8)
    g[h["top"]] = 1
    g[h["bottom"]] = 2
    ctx.set_bc([pdg.native.PD_BC_VELOCITY, pdg.native.PD_BC_FIXED], [[0.0, 5.0], [0.0, 0.0]], g)
    return ctx


def test_bond_assoc_matches_reference_default_run(pdg, hassa):
    ctx = _ctx(pdg, hassa)
    ctx.step(1)
    u, v, f = ctx.state()
    assert normwise(v, hassa["b_v1"]) < V_TOL
    assert normwise(f, hassa["b_f1"]) < F_TOL


def test_bond_assoc_matches_oracle_over_steps(pdg, po, hassa):
    dx, hor, E, nu, rho, dt = hassa["params"]
    ctx = _ctx(pdg, hassa, n1=4.0, n2=3.0)
    n = hassa["x"].shape[0]
    bc = np.zeros(n, np.uint8)
    bc[hassa["top"]] = 1
    bc[hassa["bottom"]] = 2
    sim = po.OracleSim(hassa["x"], hassa["vol"], hassa["row_ptr"], hassa["col"], E=E, nu=nu, rho=rho, dt=dt, s_c=0.0,
                       n1=4.0, n2=3.0, wlen=hor * dx, bc=bc,
                       group_kind=np.array([po.BC_VELOCITY, po.BC_FIXED], np.int32),
                       group_val=np.array([[0.0, 5.0], [0.0, 0.0]]))
    ctx.step(4)
    sim.step(4)
    u, v, f = ctx.state()
    assert normwise(u, sim.u) < 1e-12 and normwise(v, sim.v) < 1e-12 and normwise(f, sim.f) < 1e-11


@pytest.mark.parametrize("horizon", [3.2, 3.6, 4.4])
def test_bond_assoc_wide_families_match_oracle(pdg, po, horizon):
    """Families around and above 32 bonds (up to ~32, ~40 and ~61 at these
    horizons), where pass A switches from evaluating the weight matrix's lower
    triangle to per-lane rows with a partial cache: against the oracle over
    3 steps, to the same tolerance as on the reference's mesh."""
    p = pdg.plates.make_plate(26, seed=5, horizon=horizon)
    rp, col = po.build_families(p.x, p.cutoff, p.cracks)
    deg = np.diff(rp)
    assert deg.max() <= 64
    assert (deg > 32).any() and (deg <= 32).any()
    ctx = pdg.native.Context(pdg.default_params(E=p.material.E, nu=p.material.nu, rho=p.material.rho, dt=p.dt,
                                                s_c=0.0, n1=4.0, n2=3.0, weight_len=p.cutoff))
    ctx.set_particles(p.x, p.vol)
    ctx.set_families(rp, col)
    ctx.set_bc(p.group_kind, p.group_val, p.group_of)
    sim = po.OracleSim(p.x, p.vol, rp, col, E=p.material.E, nu=p.material.nu, rho=p.material.rho, dt=p.dt, s_c=0.0,
                       n1=4.0, n2=3.0, wlen=p.cutoff, bc=p.group_of, group_kind=p.group_kind, group_val=p.group_val)
    ctx.step(3)
    sim.step(3)
    u, v, f = ctx.state()
    assert normwise(u, sim.u) < 1e-12 and normwise(v, sim.v) < 1e-12 and normwise(f, sim.f) < 1e-11


def test_bond_assoc_weights_follow_set_params(pdg, hassa):
    """The per-bond weight constants (|xi|, 1/|xi|, exp(+-n1 |xi| / l)) are formed
    once per slot; pd_set_params with other weights re-forms them: a context
    switched from n1 = 4, n2 = 3 (and a longer weight length) to the reference's
    n1 = n2 = 10 steps bit for bit as one created with them."""
    dx, hor = hassa["params"][0], hassa["params"][1]
    a = _ctx(pdg, hassa, n1=4.0, n2=3.0)
    a.set_params(weight_len=1.5 * hor * dx)
    a.step(2)  # the constants formed for the first weights
    a.set_params(n1=10.0, n2=10.0, weight_len=hor * dx)
    b = _ctx(pdg, hassa)
    u, v, f = a.state()
    b.set_state(u=u, v=v, f=f)
    a.step(2)
    b.step(2)
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)


def test_bond_assoc_compute_velocity_dropin(pdg, hassa):
    """pd_compute_velocity in the bond-associated mode after the reference's host drift."""
    ctx = _ctx(pdg, hassa)
    n = hassa["x"].shape[0]
    v = np.zeros((n, 2))
    v[hassa["top"]] = [0.0, 5.0]
    u = v * hassa["params"][5]
    u[hassa["bottom"]] = 0.0
    acc = np.zeros((n, 2))
    f = ctx.compute_velocity(u, v, acc)
    assert normwise(v, hassa["b_v1"]) < V_TOL
    assert normwise(f, hassa["b_f1"]) < F_TOL


def test_bond_assoc_compute_velocity_pinned_equals_staged(pdg, hassa):
    """pd_compute_velocity in the bond-associated mode on page-locked buffers
    (what the C++ drop-in passes) against pageable buffers: bit for bit over
    three calls with the reference's drift."""
    a = _ctx(pdg, hassa)
    b = _ctx(pdg, hassa)
    n = hassa["x"].shape[0]
    dt = hassa["params"][5]
    v = np.zeros((n, 2))
    v[hassa["top"]] = [0.0, 5.0]
    u = v * dt
    u[hassa["bottom"]] = 0.0
    acc = np.zeros((n, 2))
    bufs = [pdg.native.PinnedArray((n, 2)) for _ in range(4)]
    hu, hv, ha, hf = (x.array for x in bufs)
    hu[:], hv[:], ha[:] = u, v, acc
    for _ in range(3):
        fa = a.compute_velocity(u, v, acc)
        b.compute_velocity(hu, hv, ha, netf=hf)
        assert np.array_equal(v, hv) and np.array_equal(acc, ha) and np.array_equal(fa, hf)
        u = u + v * dt + 0.5 * acc * dt ** 2
        hu[:] = u
    for x in bufs:
        x.free()


def test_bond_assoc_rejects_asymmetric_families(pdg):
    """The mode pairs every bond with its reverse: caller-supplied families in
    which 1 lists 2 but 2 does not list 1 are refused (the unmatched bond is
    made inert on the device, so nothing reads outside the families)."""
    x = np.array([[0.0, 0.0], [1e-3, 0.0], [2e-3, 0.0]])
    ctx = pdg.native.Context(pdg.default_params(s_c=0.0, n1=10.0, n2=10.0, weight_len=3e-3))
    ctx.set_particles(x, np.full(3, 1e-9))
    with pytest.raises(pdg.PdError, match="symmetric"):
        ctx.set_families(np.array([0, 1, 3, 3]), np.array([1, 0, 2]))


def test_bond_assoc_rejects_breaking_and_mixed(pdg):
    with pytest.raises(pdg.PdError):
        pdg.native.Context(pdg.default_params(n1=10.0, n2=10.0, weight_len=3.0, s_c=5e-4))
    with pytest.raises(pdg.PdError):
        pdg.native.Context(pdg.default_params(n1=10.0, n2=10.0, weight_len=3.0, precision=1))


def test_bond_assoc_step_host_equals_staged_copies(pdg, hassa):
    """pd_step_host in the bond-associated mode (the drift reads the host
    buffers, the last pass B writes them) is pd_set_state + pd_step +
    pd_get_state, bit for bit, for one step and for two."""
    a = _ctx(pdg, hassa)
    b = _ctx(pdg, hassa)
    a.step(2)
    b.step(2)
    n = hassa["x"].shape[0]
    bufs = [pdg.native.PinnedArray((n, 2)) for _ in range(3)]
    hu, hv, hf = (x.array for x in bufs)
    hu[:], hv[:], hf[:] = a.state()
    for nsteps in (1, 2):
        a.set_state(u=hu, v=hv, f=hf)
        a.step(nsteps)
        ua, va, fa = a.state()
        b.step_host(nsteps, hu, hv, hf)
        assert np.array_equal(ua, hu) and np.array_equal(va, hv) and np.array_equal(fa, hf), nsteps
    for x in bufs:
        x.free()
