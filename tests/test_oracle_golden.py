"""Pin the C restatement (oracle/pd_oracle.c) against the reference's own code.

The fixtures in tests/golden/ were produced by oracle/_ref (the reference's
main_seq.cpp + SetupParticleSystem.cpp + matrix.cpp, unmodified) after that
build reproduced the reference's shipped golden files byte for byte
(tests/golden/make_golden.py, manifest.json).

Tolerances (normwise max|d|/max|ref|): velocities and displacements 1e-10
(the parity bar); net force 1e-8 -- the reference keeps absolute
positions (~30 mm) in 80-bit long double while displacements are ~5e-9 mm,
so its own force carries ~2e-10 relative rounding, which is what we measure.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, hassa_oracle, normwise, plate_oracle

V_TOL = 1e-10
F_TOL = 1e-8


def u_tol(x, u_ref):
    """1e-10 plus the reference's own floor for displacements: it stores the
    absolute position x + u in long double (64-bit significand), so u carries
    up to half an ulp of max|x| (2**-64 * max|x|) relative to max|u|.  On the
    Hassa mesh (|x| <= 34.5 mm, u ~ 5e-9 mm after one step) that floor is
    ~4e-10; on SI plates it is ~1e-14."""
    return V_TOL + 2.0 * np.abs(x).max() * 2.0**-64 / np.abs(u_ref).max()


def test_manifest_pins_reference_goldens():
    man = json.load(open(os.path.join(GOLDEN, "manifest.json")))
    assert man["reference_golden_identical:velocity_step_0_after_seq_ref.txt"] is True
    assert man["reference_golden_identical:LocalParticlesPositions_rank_0step_0.txt"] is True
    assert man["hassa_mesh_rule_matches_reference"] is True


def test_hassa_families_match_reference(po, hassa):
    rp, col = po.build_families(hassa["x"], 1.01 * 1.0 * 3.0)
    assert np.array_equal(rp, hassa["row_ptr"])
    assert np.array_equal(col, hassa["col"])


@pytest.mark.parametrize("nth", [1, 4])
def test_hassa_classic_matches_reference(po, hassa, nth):
    sim = hassa_oracle(po, hassa)
    sim.nthreads = nth
    sim._pb.nthreads = nth
    sim.step(1)
    assert normwise(sim.v, hassa["c_v1"]) < V_TOL
    assert normwise(sim.u, hassa["c_u1"]) < u_tol(hassa["x"], hassa["c_u1"])
    assert normwise(sim.f, hassa["c_f1"]) < F_TOL
    sim.step(2)
    assert normwise(sim.v, hassa["c_v3"]) < V_TOL
    assert normwise(sim.u, hassa["c_u3"]) < u_tol(hassa["x"], hassa["c_u3"])
    assert normwise(sim.f, hassa["c_f3"]) < F_TOL


def test_plate30_families_match_reference_findneighbor(po, pdg, plate30_ref):
    p = pdg.plates.make_plate(30, seed=3, crack="centre-half")
    rp, col = po.build_families(p.x, p.cutoff)  # no crack: the reference's findNeighbor
    assert np.array_equal(rp, plate30_ref["nocrack_row_ptr"])
    assert np.array_equal(col, plate30_ref["nocrack_col"])
    deg = np.diff(rp).reshape(30, 30)
    assert deg[10:20, 10:20].min() == 28 and deg.max() == 28  # 28-offset stencil in the interior


def test_plate30_steps_match_reference(po, pdg, plate30_ref):
    p = pdg.plates.make_plate(30, seed=3, crack="centre-half")
    fam = (plate30_ref["row_ptr"], plate30_ref["col"])
    rp, col = po.build_families(p.x, p.cutoff, p.cracks)
    assert np.array_equal(rp, fam[0]) and np.array_equal(col, fam[1])
    sim = plate_oracle(po, p, s_c=0.0, families=fam, k_hg=0.0)  # the reference's model
    sim.step(1)
    assert normwise(sim.v, plate30_ref["v1"]) < V_TOL
    assert normwise(sim.u, plate30_ref["u1"]) < V_TOL
    assert normwise(sim.f, plate30_ref["f1"]) < F_TOL
    sim.step(3)
    assert normwise(sim.v, plate30_ref["v4"]) < V_TOL
    assert normwise(sim.u, plate30_ref["u4"]) < V_TOL
    assert normwise(sim.f, plate30_ref["f4"]) < F_TOL


def test_oracle_planted_mistake_is_caught(po, hassa):
    """The comparison is sharp: a 1e-6 change of E in the oracle fails it."""
    sim = hassa_oracle(po, hassa)
    sim.E = sim.E * (1 + 1e-6)
    sim._pb.E = sim.E
    sim.step(1)
    assert normwise(sim.f, hassa["c_f1"]) > F_TOL


# Mazars damage (computeDamageStatus, src/main_seq.cpp:473-598) against the
# reference run at two imposed displacement fields (tests/golden/mazars_ref.npz).
MZ_TOL = 1e-12


@pytest.fixture(scope="module")
def mazars_ref():
    return dict(np.load(os.path.join(GOLDEN, "mazars_ref.npz")))


def mazars_oracle(po, h, weights):
    dx, hor, E, nu, rho, dt = h["params"]
    return po.OracleSim(h["x"], h["vol"], h["row_ptr"], h["col"], E=E, nu=nu, rho=rho, dt=dt, n1=weights,
                        n2=weights, wlen=hor * dx)


@pytest.mark.parametrize("tag,weights", [("c", 0.0), ("b", 10.0)])
def test_mazars_matches_reference(po, hassa, mazars_ref, tag, weights):
    m = mazars_ref
    sim = mazars_oracle(po, hassa, weights)
    nnz = int(hassa["row_ptr"][-1])
    k0 = float(m["kappa0"])
    thr, bd = np.full(nnz, k0), np.zeros(nnz)
    sim.u[:] = m["u1"]
    st1 = sim.mazars(thr, bd, k0)
    assert int((thr > k0).sum()) == int(m[f"{tag}_updated1"])
    assert np.abs(st1 - m[f"{tag}_st1"]).max() < MZ_TOL
    sim.u[:] = m["u2"]
    st2 = sim.mazars(thr, bd, k0)
    assert np.abs(st2 - m[f"{tag}_st2"]).max() < MZ_TOL
    assert np.abs(thr - m[f"{tag}_thr2"]).max() < MZ_TOL * np.abs(m[f"{tag}_thr2"]).max()
    assert np.abs(bd - m[f"{tag}_bd2"]).max() < MZ_TOL
    # the fixture exercises both branches at the second call: loading and unloading bonds
    assert 0 < int((m[f"{tag}_thr2"] > k0).sum()) < nnz and 0.2 < m[f"{tag}_st2"].mean() < 0.9
