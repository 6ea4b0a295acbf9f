"""Serving loop: continuous batching with admission by HBM footprint; every
request's result equals the same request run alone (bit for bit)."""
import numpy as np
import pytest


def test_request_stream_is_seeded_and_bounded(pdg):
    serve = pdg.serve if hasattr(pdg, "serve") else __import__("importlib").import_module("2d_pd_gpu_gb300.serve")
    a = serve.make_requests(200, seed=3, rate=10.0)
    b = serve.make_requests(200, seed=3, rate=10.0)
    assert [(q.nx, q.ny, q.steps, q.arrival) for q in a] == [(q.nx, q.ny, q.steps, q.arrival) for q in b]
    n = np.array([q.particles for q in a])
    assert n.min() >= 0.8e4 and n.max() <= 2.2e6
    assert all(q.nx in (q.ny, 2 * q.ny) for q in a)
    assert all(200 <= q.steps <= 2000 for q in a)
    arr = np.array([q.arrival for q in a])
    assert np.all(np.diff(arr) >= 0) and 5.0 < arr[-1] < 40.0  # ~200 / 10 per s


def test_footprint_admission_math(pdg):
    serve = __import__("importlib").import_module("2d_pd_gpu_gb300.serve")
    f64 = serve.footprint(2_000_000, pdg.native.PD_FP64)
    mix = serve.footprint(2_000_000, pdg.native.PD_MIXED)
    assert 2e9 < f64 < 5e9 and 0.5e9 < mix < 1.5e9  # per 2M-particle plate


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("mode", [0, 2])  # phase kernels; per-member graphs (the default)
def test_served_results_equal_solo(pdg, precision, mode):
    serve = __import__("importlib").import_module("2d_pd_gpu_gb300.serve")
    reqs = serve.make_requests(10, seed=7, lo=2e3, hi=6e4, steps_lo=20, steps_hi=120, rate=400.0)
    # a budget that forces some requests to wait for memory
    budget = 2.5 * max(serve.footprint(q.particles, precision) for q in reqs)
    cfg = dict(persistent=mode, block=256, tile=256, blocks_per_sm=1)
    srv = serve.Server(precision=precision, budget_bytes=budget, max_plates=4, chunk=16, workers=2,
                       batch_config=cfg)
    m = srv.run(reqs)
    assert m["requests"] == len(reqs)
    assert m["p99_latency_s"] >= m["p50_latency_s"] > 0
    by = {r.rid: r for r in srv.results}
    for q in reqs[::3]:
        d, broken = serve.solo_digest(q, precision)
        assert by[q.rid].digest == d, f"request {q.rid} differs alone vs in the mix"
        assert by[q.rid].broken == broken


@pytest.mark.gpu
def test_preemption_by_checkpoint_keeps_results(pdg):
    """A long request holds the memory budget when short ones arrive: it is
    checkpointed to host memory, the short ones run, and it resumes; every
    result still equals its solo run bit for bit."""
    serve = __import__("importlib").import_module("2d_pd_gpu_gb300.serve")
    mat = pdg.plates.Material()
    big = serve.Request(0, 0.0, 160, 160, 2000, 11, mat, 1.0, None)
    small = [serve.Request(k, 0.01 * k, 48, 48, 30, 11 + k, mat, 1.5, None) for k in (1, 2, 3)]
    reqs = [big] + small
    f = lambda q: serve.footprint(q.particles, pdg.native.PD_MIXED)
    budget = f(big) + 0.5 * f(small[0])
    srv = serve.Server(precision=pdg.native.PD_MIXED, budget_bytes=budget, max_plates=4, chunk=10, workers=2)
    m = srv.run(reqs)
    assert m["requests"] == 4 and m["preemptions"] >= 1
    by = {r.rid: r for r in srv.results}
    assert by[0].finished > max(by[k].finished for k in (1, 2, 3))  # the short ones overtook it
    for q in reqs:
        d, broken = serve.solo_digest(q, pdg.native.PD_MIXED)
        assert by[q.rid].digest == d and by[q.rid].broken == broken
