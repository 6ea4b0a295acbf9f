"""The zero-energy-mode penalty against hand calculations.

The penalty adds T_ij = k (d_ij - G_i xi_ij) (omega = 1) to every bond, so
f_i gains 2k sum_j V_j d_ij - k G_i sum_j V_j xi_ij - k sum_j V_j G_j xi_ij
(d: relative displacement, G = D K^-1 = F - I).  It is linear in k and
independent of the stress, so f(k) - f(0) isolates it.  Two closed forms on a
perfect square grid (no jitter, no crack, no breaking), horizon 3.015 dx:

* an affine field u = H x: G_i = H wherever K_i is invertible and
  d_ij = H xi_ij, so every bond's non-affine part is zero and the penalty
  force vanishes at every particle, boundary rows included;
* one interior particle p displaced by delta, every other particle at rest:
  sum_j V_j xi_pj = 0 and K_j = kappa I for p and its neighbours (full
  families, symmetric under quarter turns), so G_p = 0,
  G_j xi_pj = -V delta |xi_pj|^2 / kappa and sum_j V |xi_pj|^2 = 2 kappa,
  which gives f_p(k) - f_p(0) = -2 k V delta (N - 1) with N = |family(p)|.

The oracle (CPU) and the GPU forms are checked against both.
"""
import numpy as np
import pytest

import importlib

plates = importlib.import_module("2d_pd_gpu_gb300.plates")

SIDE = 21
K_HG = 3.0e24  # N / m^6, the plate workloads' order of magnitude
DELTA = np.array([7.0e-7, -3.0e-7])
H = np.array([[1.0e-4, 2.0e-5], [-3.0e-5, 5.0e-5]])


def _grid():
    p = plates.make_plate(SIDE, jitter=0.0)
    p.material.s_c = 0.0
    return p


def _fields(p):
    centre = (SIDE // 2) * SIDE + SIDE // 2
    assert np.allclose(p.x[centre], 0.0)
    u_point = np.zeros((p.n, 2))
    u_point[centre] = DELTA
    u_affine = p.x @ H.T
    return centre, u_point, u_affine


def _oracle_force(po, p, rp, col, u, k):
    sim = po.OracleSim(p.x, p.vol, rp, col, E=p.material.E, nu=p.material.nu, rho=p.material.rho, dt=p.dt,
                       s_c=0.0, k_hg=k)
    sim.u[:] = u
    sim.step(1)  # v = f = 0 and no BC groups: the drift leaves u as set, pass B gives f(u)
    assert np.array_equal(sim.u, u)
    return sim.f.copy()


def test_oracle_penalty_closed_forms(po):
    p = _grid()
    rp, col = po.build_families(p.x, p.cutoff, p.cracks)
    centre, u_point, u_affine = _fields(p)
    n_fam = int(rp[centre + 1] - rp[centre])
    assert n_fam == 28
    vol = p.vol[0]
    df = _oracle_force(po, p, rp, col, u_point, K_HG) - _oracle_force(po, p, rp, col, u_point, 0.0)
    expect = -2.0 * K_HG * vol * DELTA * (n_fam - 1)
    assert np.abs(df[centre] - expect).max() <= 1e-12 * np.abs(expect).max()
    # the affine field: zero to rounding, against the size of one bond's penalty term times the family
    df = _oracle_force(po, p, rp, col, u_affine, K_HG) - _oracle_force(po, p, rp, col, u_affine, 0.0)
    scale = K_HG * vol * np.abs(H).max() * p.dx * n_fam
    assert np.abs(df).max() <= 1e-10 * scale


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol_point,tol_affine", [(0, 1e-12, 1e-10), (1, 2e-6, 2e-5)])
def test_gpu_penalty_closed_forms(pdg, precision, tol_point, tol_affine):
    """FP64 form to rounding; the mixed form (FP32 bond arithmetic) to its
    single-precision accuracy."""
    p = _grid()
    centre, u_point, u_affine = _fields(p)

    def force(u, k):
        c = p.context(precision=precision, k_hg=k)
        c.set_bc([pdg.native.PD_BC_NONE], [[0.0, 0.0]], np.zeros(p.n, np.uint8))
        c.set_state(u=u, v=np.zeros_like(u), f=np.zeros_like(u))
        c.step(1)
        f = c.state()[2]
        c.close()
        return f

    fam = None
    vol = p.vol[0]
    df = force(u_point, K_HG) - force(u_point, 0.0)
    import pd_oracle as po

    rp, _ = po.build_families(p.x, p.cutoff, p.cracks)
    fam = int(rp[centre + 1] - rp[centre])
    expect = -2.0 * K_HG * vol * DELTA * (fam - 1)
    assert np.abs(df[centre] - expect).max() <= tol_point * np.abs(expect).max()
    df = force(u_affine, K_HG) - force(u_affine, 0.0)
    scale = K_HG * vol * np.abs(H).max() * p.dx * fam
    assert np.abs(df).max() <= tol_affine * scale
