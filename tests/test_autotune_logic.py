"""The autotuner's host logic (candidate timing, refused configurations,
the per-GPU cache) against a stand-in batch whose step time is a known
function of the launch shape: no GPU."""
import importlib
import json

import pytest

autotune = importlib.import_module("2d_pd_gpu_gb300.autotune")
native = importlib.import_module("2d_pd_gpu_gb300.native")


def cost(cfg):
    """ms per step of a launch shape (the stand-in's ground truth)."""
    return 1.0 + 0.3 * cfg["persistent"] + abs(cfg["block"] - 256) / 512 + abs(cfg["tile"] - 1024) / 8192 \
        + 0.05 * cfg.get("blocks_per_sm", 1)


class FakeBatch:
    def __init__(self, precision=native.PD_FP64, refuse=()):
        self.precision = precision
        self.cfg = None
        self.refuse = [json.dumps(c, sort_keys=True) for c in refuse]
        self.timed = 0
        self.closed = False

    def info(self):
        return {"particles": 3_000_000, "plates": 200, "bonds": 84_000_000}

    def set_config(self, **cfg):
        if json.dumps(cfg, sort_keys=True) in self.refuse:
            raise native.PdError(-1, "refused")
        self.cfg = cfg

    def step(self, k):
        pass

    def synchronize(self):
        pass

    def step_timed(self, k):
        self.timed += 1
        return cost(self.cfg) * k

    def close(self):
        self.closed = True


class FakeCtx:
    def __init__(self):
        self.closed = False

    def close(self):
        self.closed = True


def test_tune_batch_picks_the_fastest_and_skips_refused():
    cands = autotune.candidates_for(native.PD_FP64)
    best_true = min(cands, key=cost)
    b = FakeBatch(refuse=[best_true])
    best, timings = autotune.tune_batch(b, candidates=cands)
    rest = [c for c in cands if c != best_true]
    assert best == min(rest, key=cost)
    assert json.dumps(best_true, sort_keys=True) not in timings and len(timings) == len(rest)
    assert b.cfg == best  # left at the winner


def test_tune_batch_with_nothing_running_raises():
    cands = autotune.candidates_for(native.PD_MIXED)
    with pytest.raises(RuntimeError):
        autotune.tune_batch(FakeBatch(native.PD_MIXED, refuse=cands), candidates=cands)


def test_tune_caches_per_gpu_precision_and_size(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "autotune.json"))
    made = []

    def make():
        b, ctxs = FakeBatch(), [FakeCtx(), FakeCtx()]
        made.append((b, ctxs))
        return b, ctxs

    best1, t1 = autotune.tune(make, native.PD_FP64)
    best2, t2 = autotune.tune(make, native.PD_FP64)
    assert best1 == best2 == min(autotune.candidates_for(native.PD_FP64), key=cost) and t1 == t2
    assert made[0][0].timed > 0 and made[1][0].timed == 0  # the second call came from the cache
    for b, ctxs in made:  # the throwaway batches and their contexts are released
        assert b.closed and all(c.closed for c in ctxs)
    cache = json.load(open(tmp_path / "autotune.json"))
    assert len(cache) == 1 and next(iter(cache)).endswith("|" + autotune.bucket(FakeBatch().info()))
    autotune.tune(make, native.PD_MIXED)  # another precision: another entry
    assert len(json.load(open(tmp_path / "autotune.json"))) == 2


def test_size_buckets():
    assert autotune.bucket({"particles": 1 << 20, "plates": 256}) == "p20-n8"
    assert autotune.bucket({"particles": 0, "plates": 0}) == "p0-n0"
