"""Batched ragged plates (pd_batch): one persistent cooperative kernel (or a
graph of phase kernels) steps every member; each plate's result must equal
its solo run bit for bit, whatever the mix and the tuning."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPECS = [(37, 1), (64, 2), (20, 3), (51, 4), (96, 5)]


def _plates(pdg):
    out = []
    for side, seed in SPECS:
        p = pdg.plates.make_plate(side, seed=seed, crack="centre-half")
        p.material.s_c = 2e-4  # breaks bonds within the short runs
        out.append(p)
    return out


def _solo(pdg, plates, precision, steps):
    res = []
    for p in plates:
        c = p.context(precision=precision)
        c.step(steps)
        res.append((*c.state(), c.bond_mask(), c.damage()))
        c.close()
    return res


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("cfg", [dict(persistent=1, block=256, tile=1024, blocks_per_sm=2),
                                 dict(persistent=1, block=128, tile=256, blocks_per_sm=1),
                                 dict(persistent=0, block=256, tile=512, blocks_per_sm=1),
                                 dict(persistent=2, block=256, tile=256, blocks_per_sm=1)])
def test_batch_equals_solo(pdg, precision, cfg):
    plates = _plates(pdg)
    steps = 23
    solo = _solo(pdg, plates, precision, steps)
    b = pdg.Batch(precision=precision)
    b.set_config(**cfg)
    ctxs = [p.context(precision=precision) for p in plates]
    for c in ctxs:
        b.add(c)
    info = b.info()
    assert info["plates"] == len(plates) and info["particles"] == sum(p.n for p in plates)
    b.step(10)
    b.step(13)  # two calls: state carries across, first call's graph reused for nothing
    b.synchronize()
    broke = 0
    for c, ref in zip(ctxs, solo):
        got = (*c.state(), c.bond_mask(), c.damage())
        for g, r in zip(got, ref):
            assert np.array_equal(g, r)
        broke += int((ref[3] == 0).sum())
        assert c.counters()["steps"] == steps
    assert broke > 0


@pytest.mark.parametrize("mode", [1, 2])  # the persistent kernel; per-member graphs (the default)
def test_batch_membership_changes(pdg, mode):
    """Continuous batching: members join and leave between steps; everyone's
    trajectory is still its solo trajectory."""
    plates = _plates(pdg)
    solo = _solo(pdg, plates, 0, 20)
    b = pdg.Batch(precision=0)
    b.set_config(persistent=mode)
    ctxs = [p.context() for p in plates]
    b.add(ctxs[0])
    b.add(ctxs[1])
    b.step(5)  # 0,1 at 5
    b.add(ctxs[2])
    b.step(5)  # 0,1 at 10; 2 at 5
    b.remove(ctxs[0])
    ctxs[0].step(10)  # 0 finishes alone
    b.add(ctxs[3])
    b.add(ctxs[4])
    b.step(10)  # 1 at 20, 2 at 15, 3,4 at 10
    b.remove(ctxs[1])
    b.step(5)  # 2 at 20, 3,4 at 15
    b.remove(ctxs[2])
    b.step(5)  # 3,4 at 20
    b.synchronize()
    for c, ref in zip(ctxs, solo):
        assert c.counters()["steps"] == 20
        for g, r in zip((*c.state(), c.bond_mask(), c.damage()), ref):
            assert np.array_equal(g, r)
    ctxs[3].close()  # pd_destroy leaves the batch
    assert b.info()["plates"] == 1
    b.step(1)
    b.synchronize()


def test_batch_rejects_mixed_precisions(pdg):
    p = pdg.plates.make_plate(16, seed=1)
    b = pdg.Batch(precision=0)
    with pytest.raises(pdg.PdError):
        b.add(p.context(precision=1))


@pytest.mark.parametrize("precision", [0, 1])
def test_barrier_wait_runs_out_and_the_batch_recovers(pdg, precision):
    """A bounded device wait that runs out, without any fault: block 0 of the
    persistent kernel holds 2 ms before every grid barrier while the others
    may poll 16 times, so their waits give up; every block returns (the
    kernel ends, the stream stays usable), pd_batch_synchronize reports
    PD_ERR_TIMEOUT, and after pd_reset the same batch steps bit-identically
    to the solo runs."""
    plates = _plates(pdg)
    steps = 5
    solo = _solo(pdg, plates, precision, steps)
    b = pdg.Batch(precision=precision)
    b.set_config(persistent=1, block=256, tile=256, blocks_per_sm=1)
    ctxs = [p.context(precision=precision) for p in plates]
    for c in ctxs:
        b.add(c)
    b.set_barrier_limits(spin_limit=16, hold_ns=2_000_000)
    b.step(3)
    with pytest.raises(pdg.native.PdError) as err:
        b.synchronize()
    assert err.value.code == -7 and "grid-barrier" in str(err.value)
    b.set_barrier_limits(0, 0)
    for c in ctxs:
        c.reset()
    b.step(steps)
    b.synchronize()
    for c, ref in zip(ctxs, solo):
        got = (*c.state(), c.bond_mask(), c.damage())
        for g, r in zip(got, ref):
            assert np.array_equal(g, r)
    b.close()
    for c in ctxs:
        c.close()
