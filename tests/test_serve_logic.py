"""The serving loop's host logic (admission by footprint, contexts built
ahead of admission, preemption by checkpoint, retirement while the next
chunk runs) against a stand-in batch and stand-in contexts: no GPU.  The
stand-ins count steps and device bytes, so the tests check that every
request runs exactly its steps, that FIFO order holds, and that the bytes
held never exceed the budget."""
import importlib
import threading

import numpy as np
import pytest

serve = importlib.import_module("2d_pd_gpu_gb300.serve")
native = importlib.import_module("2d_pd_gpu_gb300.native")


class Ledger:
    """Device bytes held by live stand-in contexts, and the peak."""

    def __init__(self):
        self.lock = threading.Lock()
        self.live = 0.0
        self.peak = 0.0

    def take(self, b):
        with self.lock:
            self.live += b
            self.peak = max(self.peak, self.live)

    def give(self, b):
        with self.lock:
            self.live -= b


class FakeCtx:
    def __init__(self, request, precision, ledger):
        self.request = request
        self.n = request.particles
        self.nnz = 28 * self.n
        self.steps = 0
        self.bytes = serve.footprint(self.n, precision)
        self.ledger = ledger
        ledger.take(self.bytes)
        self.closed = False

    def state(self):
        u = np.full((self.n, 2), float(self.steps))
        return u, u.copy(), u.copy()

    def bond_mask(self):
        return np.ones(self.nnz, dtype=np.uint8)

    def checkpoint(self):
        return self.steps.to_bytes(8, "little")

    def restore(self, blob):
        self.steps = int.from_bytes(blob, "little")

    def close(self):
        assert not self.closed
        self.closed = True
        self.ledger.give(self.bytes)


class FakePlate:
    def __init__(self, request, ledger):
        self.request = request
        self.ledger = ledger

    def context(self, precision, device=0):
        return FakeCtx(self.request, precision, self.ledger)


class FakeBatch:
    log = []

    def __init__(self, precision, device=0):
        self.members = []

    def set_config(self, **kw):
        pass

    def add(self, ctx):
        assert ctx not in self.members and not ctx.closed
        self.members.append(ctx)
        FakeBatch.log.append(("add", ctx.request.rid))

    def remove(self, ctx):
        self.members.remove(ctx)

    def step(self, k):
        for c in self.members:
            c.steps += k
            assert c.steps <= c.request.steps, "a request ran past its step count"

    def synchronize(self):
        pass

    def last_step_ms(self):
        return 0.01

    def close(self):
        pass


@pytest.fixture
def fake(monkeypatch):
    ledger = Ledger()
    FakeBatch.log = []
    monkeypatch.setattr(native, "Batch", FakeBatch)
    monkeypatch.setattr(serve.Request, "plate", lambda self: FakePlate(self, ledger))
    return ledger


def _requests(count, seed, rate=None):
    return serve.make_requests(count, seed=seed, lo=2e3, hi=6e4, steps_lo=20, steps_hi=120, rate=rate)


def _ran_exactly(srv, reqs, ledger):
    """Every result's digest is that of a context that took exactly its request's steps."""
    by = {r.rid: r for r in srv.results}
    assert sorted(by) == sorted(q.rid for q in reqs)
    for q in reqs:
        c = FakeCtx(q, native.PD_MIXED, ledger)
        c.steps = q.steps
        assert by[q.rid].digest == serve.state_digest(c)[0], f"request {q.rid} ran a wrong number of steps"
        c.close()


pytestmark = pytest.mark.timeout(120)


@pytest.mark.parametrize("precision", [native.PD_FP64, native.PD_MIXED])
def test_every_request_runs_its_steps_under_the_budget(fake, precision):
    reqs = _requests(24, seed=5)
    budget = 3.0 * max(serve.footprint(q.particles, precision) for q in reqs)
    srv = serve.Server(precision=precision, budget_bytes=budget, max_plates=6, chunk=16, workers=3, preempt=False)
    m = srv.run(reqs)
    assert m["requests"] == len(reqs)
    _ran_exactly(srv, reqs, fake)
    by = {r.rid: r for r in srv.results}
    for q in reqs:
        assert by[q.rid].finished >= by[q.rid].admitted >= q.arrival
    assert fake.peak <= budget + 1e-6, "contexts held more device memory than the budget"
    assert fake.live == 0.0  # every context closed
    adds = [rid for op, rid in FakeBatch.log if op == "add"]
    assert adds == sorted(adds)  # FIFO admission (arrival order = request order here)


def test_preemption_parks_and_resumes(fake):
    mat = serve.plates.Material()
    big = serve.Request(0, 0.0, 160, 160, 2000, 11, mat, 1.0, None)
    small = [serve.Request(k, 0.0, 48, 48, 30, 11 + k, mat, 1.5, None) for k in (1, 2, 3)]
    f = lambda q: serve.footprint(q.particles, native.PD_MIXED)
    budget = f(big) + 0.5 * f(small[0])
    srv = serve.Server(precision=native.PD_MIXED, budget_bytes=budget, max_plates=4, chunk=10, workers=2)
    m = srv.run([big] + small)
    assert m["requests"] == 4 and m["preemptions"] >= 1
    _ran_exactly(srv, [big] + small, fake)
    by = {r.rid: r for r in srv.results}
    # the short requests finished before the long one, which resumed from its checkpoint
    assert max(by[k].finished for k in (1, 2, 3)) <= by[0].finished
    assert fake.live == 0.0


def test_a_request_larger_than_the_budget_still_runs_alone(fake):
    reqs = _requests(4, seed=9)
    budget = 0.5 * min(serve.footprint(q.particles, native.PD_MIXED) for q in reqs)
    srv = serve.Server(precision=native.PD_MIXED, budget_bytes=budget, max_plates=4, chunk=25, workers=2,
                       preempt=False)
    m = srv.run(reqs)
    assert m["requests"] == len(reqs)
    # one at a time: never more than the largest single footprint held
    assert fake.peak <= max(serve.footprint(q.particles, native.PD_MIXED) for q in reqs) + 1e-6


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_stream_with_preemption_finishes_within_the_budget(fake, seed):
    """A Poisson stream with preemption on: no deadlock, every request runs
    exactly its steps (across checkpoints), the budget holds."""
    reqs = serve.make_requests(40, seed=seed, lo=2e3, hi=6e4, steps_lo=20, steps_hi=400, rate=2000.0)
    budget = 2.5 * max(serve.footprint(q.particles, native.PD_MIXED) for q in reqs)
    srv = serve.Server(precision=native.PD_MIXED, budget_bytes=budget, max_plates=5, chunk=8, workers=3,
                       preempt=True, preempt_ratio=2.0)
    m = srv.run(reqs)
    assert m["requests"] == len(reqs)
    _ran_exactly(srv, reqs, fake)
    assert fake.peak <= budget + 1e-6
    assert fake.live == 0.0
