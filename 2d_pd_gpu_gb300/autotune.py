"""Autotuner for batched stepping (pd_batch launch shape).

Chooses, by measurement on this GPU, the launch mode (one persistent
cooperative kernel, a graph of phase kernels, or every plate's own
single-plate kernels on one stream per plate), threads per block,
particles per work tile, and persistent blocks per SM.  Mixed-form batches
always run 256-thread blocks over the plates' visiting blocks (the
shared-memory halo code of the single-plate passes), so for them only the
launch mode and blocks per SM are searched.  The tuning never changes the
arithmetic (one thread owns one particle at a time, and the per-particle
code is the same), so a plate's results do not depend on the chosen
configuration -- tests/test_gpu_batch.py checks that bit for bit.

Candidates are timed on a throwaway batch built from the same plates (the
caller passes a factory), so tuning does not advance the real simulation.
Results are cached in 2d_pd_gpu_gb300/_build/autotune.json, keyed by GPU,
precision and a coarse size bucket.
"""
from __future__ import annotations

import json
import math
import os
import threading

from . import native

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")
_lock = threading.Lock()

CANDIDATES = (
    [dict(persistent=1, block=b, tile=t, blocks_per_sm=s) for b in (128, 256) for t in (256, 1024, 4096)
     for s in (1, 2, 4)]
    + [dict(persistent=0, block=b, tile=t, blocks_per_sm=1) for b in (128, 256) for t in (256, 1024)]
    + [dict(persistent=2, block=256, tile=256, blocks_per_sm=1)]
)
MIXED_CANDIDATES = ([dict(persistent=1, block=256, tile=256, blocks_per_sm=s) for s in (1, 2, 3, 4)]
                    + [dict(persistent=0, block=256, tile=256, blocks_per_sm=1)]
                    + [dict(persistent=2, block=256, tile=256, blocks_per_sm=1)])


def candidates_for(precision):
    return MIXED_CANDIDATES if precision == native.PD_MIXED else CANDIDATES


def _gpu_name(device):
    try:
        import torch

        return torch.cuda.get_device_name(device)
    except Exception:
        return f"device{device}"


def bucket(info):
    """Coarse size bucket: log2 of particles and of plate count."""
    return f"p{int(math.log2(max(info['particles'], 1)))}-n{int(math.log2(max(info['plates'], 1)))}"


def _load():
    try:
        return json.load(open(CACHE))
    except Exception:
        return {}


def _save(d):
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + ".tmp"
    json.dump(d, open(tmp, "w"), indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def tune(make_batch, precision, device=0, steps=4, warmup=2, candidates=None, use_cache=True):
    """make_batch() -> (Batch, [contexts]) built from the workload's plates.
    Returns (best_config, {config_key: ms_per_step})."""
    candidates = candidates_for(precision) if candidates is None else candidates
    probe, ctxs = make_batch()
    info = probe.info()
    key = f"{_gpu_name(device)}|{precision}|{bucket(info)}"
    with _lock:
        cache = _load() if use_cache else {}
    if use_cache and key in cache:
        for c in ctxs:
            c.close()
        probe.close()
        return cache[key]["best"], cache[key]["timings"]
    timings = {}
    best, best_ms = None, math.inf
    for cfg in candidates:
        try:
            probe.set_config(**cfg)
            probe.step(warmup)
            probe.synchronize()
            ms = probe.step_timed(steps) / steps
        except native.PdError:
            continue
        timings[json.dumps(cfg, sort_keys=True)] = ms
        if ms < best_ms:
            best, best_ms = cfg, ms
    for c in ctxs:
        c.close()
    probe.close()
    if best is None:
        raise RuntimeError("autotune: no candidate configuration ran")
    if use_cache:
        with _lock:
            cache = _load()
            cache[key] = {"best": best, "timings": timings, "particles": info["particles"], "plates": info["plates"]}
            _save(cache)
    return best, timings


def tune_batch(batch, steps=3, warmup=1, candidates=None):
    """Measure the candidates on `batch` itself (this advances its plates:
    reset them afterwards).  Returns (best_config, {config_key: ms_per_step})
    and leaves the batch set to the best configuration."""
    candidates = candidates_for(batch.precision) if candidates is None else candidates
    timings = {}
    best, best_ms = None, math.inf
    for cfg in candidates:
        try:
            batch.set_config(**cfg)
            batch.step(warmup)
            batch.synchronize()
            ms = batch.step_timed(steps) / steps
        except native.PdError:
            continue
        timings[json.dumps(cfg, sort_keys=True)] = ms
        if ms < best_ms:
            best, best_ms = cfg, ms
    if best is None:
        raise RuntimeError("autotune: no candidate configuration ran")
    batch.set_config(**best)
    return best, timings
