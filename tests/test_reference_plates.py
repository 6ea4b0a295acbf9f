"""The benchmark plates against the reference's OWN sequential step.

tests/golden/config1_ref.npz and plate200_ref.npz come from oracle/_ref (the
reference's src/main_seq.cpp + SetupParticleSystem.cpp + matrix.cpp, driven
in its step order src/main_seq.cpp:680-715 by oracle/ref_harness.cpp) with the
reference's model: no zero-energy-mode penalty (k_hg = 0), no bond breaking
(s_c = 0), families cut by the pre-crack (tests/golden/make_golden.py, step 6):

- the config-1 plate (100 x 100, seed 0, centre half-width crack) for 3 steps
  from rest, and for 3 steps from a seeded preloaded state in which every
  particle is displaced and moving (so the crack faces and the whole interior
  carry load from the first step, not only the rows the loading wave reaches);
- the 200 x 200 cut of the 1M-particle workload (config_plate_scale(side=200,
  seed=0)) for 2 steps from rest.

Bars (normwise max|d| / max|ref|): displacements and velocities 1e-10, net
force 1e-8 (the reference's long-double force carries ~2e-10 of its own
rounding).  The oracle (CPU) and the FP64 CUDA path (GPU, through the C ABI)
are held to the same bars; the mixed form is held to its 1e-6 displacement bar
against the same reference run.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, normwise, plate_oracle
from test_oracle_golden import F_TOL, V_TOL

sys.path.insert(0, GOLDEN)
import make_golden  # noqa: E402  (preload_state, families_sha: the generator's own definitions)

MIXED_U_TOL = 1e-6


@pytest.fixture(scope="module")
def config1_ref():
    return dict(np.load(os.path.join(GOLDEN, "config1_ref.npz")))


@pytest.fixture(scope="module")
def plate200_ref():
    return dict(np.load(os.path.join(GOLDEN, "plate200_ref.npz")))


def _check(u, v, f, ref, key):
    eu, ev, ef = normwise(u, ref[f"{key[0]}_u{key[1]}"]), normwise(v, ref[f"{key[0]}_v{key[1]}"]), \
        normwise(f, ref[f"{key[0]}_f{key[1]}"])
    assert eu < V_TOL and ev < V_TOL and ef < F_TOL, f"{key}: u {eu:.2e} v {ev:.2e} f {ef:.2e}"
    return eu, ev, ef


def _preload(p, ref):
    u0, v0 = make_golden.preload_state(p)
    assert make_golden.state_sha(u0, v0) == str(ref["state_sha"]), "preloaded state regenerated differently"
    return u0, v0


# ------------------------------------------------------------------ oracle (CPU)

def test_oracle_config1_families_are_the_fixtures(po, pdg, config1_ref):
    p = pdg.plates.config_plate_100(seed=0)
    rp, col = po.build_families(p.x, p.cutoff, p.cracks)
    assert make_golden.families_sha(rp, col) == str(config1_ref["families_sha"])


def test_oracle_config1_from_rest_matches_reference(po, pdg, config1_ref):
    p = pdg.plates.config_plate_100(seed=0)
    sim = plate_oracle(po, p, s_c=0.0, k_hg=0.0)
    sim.step(1)
    _check(sim.u, sim.v, sim.f, config1_ref, ("rest", 1))
    sim.step(2)
    _check(sim.u, sim.v, sim.f, config1_ref, ("rest", 3))


def test_oracle_config1_preloaded_matches_reference(po, pdg, config1_ref):
    p = pdg.plates.config_plate_100(seed=0)
    sim = plate_oracle(po, p, s_c=0.0, k_hg=0.0)
    sim.u[:], sim.v[:] = _preload(p, config1_ref)
    sim.step(3)
    _check(sim.u, sim.v, sim.f, config1_ref, ("pre", 3))
    # the preloaded run loads every particle: no exact zeros left in the force
    assert (np.abs(config1_ref["pre_f3"]).max(axis=1) > 0).all()


def test_oracle_plate200_matches_reference(po, pdg, plate200_ref):
    p = pdg.plates.config_plate_scale(side=200, seed=0)
    rp, col = po.build_families(p.x, p.cutoff, p.cracks)
    assert make_golden.families_sha(rp, col) == str(plate200_ref["families_sha"])
    sim = plate_oracle(po, p, s_c=0.0, k_hg=0.0, families=(rp, col))
    sim.step(1)
    _check(sim.u, sim.v, sim.f, plate200_ref, ("rest", 1))
    sim.step(1)
    _check(sim.u, sim.v, sim.f, plate200_ref, ("rest", 2))


def test_oracle_planted_mistake_fails_config1(po, pdg, config1_ref):
    """The bar is sharp on this fixture too: nu off by 1e-7 fails it."""
    p = pdg.plates.config_plate_100(seed=0)
    sim = plate_oracle(po, p, s_c=0.0, k_hg=0.0)
    sim._pb.nu = sim.nu * (1 + 1e-7)
    sim.u[:], sim.v[:] = _preload(p, config1_ref)
    sim.step(3)
    assert normwise(sim.f, config1_ref["pre_f3"]) > F_TOL


# -------------------------------------------------------- CUDA path (GPU, C ABI)

@pytest.mark.gpu
def test_gpu_config1_from_rest_matches_reference(pdg, config1_ref):
    p = pdg.plates.config_plate_100(seed=0)
    ctx = p.context(s_c=0.0, k_hg=0.0)  # the reference's model
    assert make_golden.families_sha(*ctx.families()) == str(config1_ref["families_sha"])
    ctx.step(1)
    _check(*ctx.state(), config1_ref, ("rest", 1))
    ctx.step(2)
    _check(*ctx.state(), config1_ref, ("rest", 3))
    ctx.close()


@pytest.mark.gpu
def test_gpu_config1_preloaded_matches_reference(pdg, config1_ref):
    p = pdg.plates.config_plate_100(seed=0)
    ctx = p.context(s_c=0.0, k_hg=0.0)
    u0, v0 = _preload(p, config1_ref)
    ctx.set_state(u0, v0, np.zeros_like(u0))
    ctx.step(3)
    _check(*ctx.state(), config1_ref, ("pre", 3))
    ctx.close()


@pytest.mark.gpu
def test_gpu_config1_preloaded_through_step_host_matches_reference(pdg, config1_ref):
    """The end-to-end host-buffer call reaches the same reference result."""
    p = pdg.plates.config_plate_100(seed=0)
    ctx = p.context(s_c=0.0, k_hg=0.0)
    u0, v0 = _preload(p, config1_ref)
    bufs = [pdg.native.PinnedArray((p.n, 2)) for _ in range(3)]
    bufs[0].array[:], bufs[1].array[:], bufs[2].array[:] = u0, v0, 0.0
    for _ in range(3):
        ctx.step_host(1, bufs[0].array, bufs[1].array, bufs[2].array)
    _check(bufs[0].array.copy(), bufs[1].array.copy(), bufs[2].array.copy(), config1_ref, ("pre", 3))
    for b in bufs:
        b.free()
    ctx.close()


@pytest.mark.gpu
def test_gpu_plate200_matches_reference(pdg, plate200_ref):
    p = pdg.plates.config_plate_scale(side=200, seed=0)
    ctx = p.context(s_c=0.0, k_hg=0.0)
    assert make_golden.families_sha(*ctx.families()) == str(plate200_ref["families_sha"])
    ctx.step(1)
    _check(*ctx.state(), plate200_ref, ("rest", 1))
    ctx.step(1)
    _check(*ctx.state(), plate200_ref, ("rest", 2))
    ctx.close()


@pytest.mark.gpu
def test_gpu_mixed_config1_preloaded_within_bar_of_reference(pdg, config1_ref):
    p = pdg.plates.config_plate_100(seed=0)
    ctx = p.context(precision=pdg.native.PD_MIXED, s_c=0.0, k_hg=0.0)
    u0, v0 = _preload(p, config1_ref)
    ctx.set_state(u0, v0, np.zeros_like(u0))
    ctx.step(3)
    u, v, _ = ctx.state()
    assert normwise(u, config1_ref["pre_u3"]) < MIXED_U_TOL
    assert normwise(v, config1_ref["pre_v3"]) < MIXED_U_TOL
    ctx.close()
