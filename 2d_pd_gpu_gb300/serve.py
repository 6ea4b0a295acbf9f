"""Serving loop: continuous batching of fracture-solve requests on one GPU.

Requests (plate size, crack, material, load, step count) arrive over time.
A request is admitted when its estimated HBM footprint fits under the budget
and a batch slot is free; its plate is then built on the GPU (families by
the cell list, spatial layout) on a builder thread while the GPU steps the
batch, kept resident, and joins the running pd_batch, so its steps overlap
with everyone else's.  The loop advances all active requests
together in chunks (never past any request's remaining step count), retires
finished requests from the batch between chunks and reads their results
(and frees their memory) while the next chunk runs, and admits waiting ones
as memory and slots free up.  Host-side plate generation runs on worker
threads ahead of admission.

Because every plate's arithmetic is independent of the batch it runs in, a
request's result is the same alone and in the mix (bit for bit, FP64 and
mixed alike; tests/test_gpu_serve.py).

Reported: per-request latency (completion - arrival) p50/p99/mean, queueing
delay, aggregate bond-updates/s over the makespan.
"""
from __future__ import annotations

import hashlib
import math
import time
from collections import deque
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from . import native, plates

# bytes per particle and per bond slot actually allocated (pd_api.cu): state,
# geometry, staging, CSR, SELL and per-bond data; the mixed form adds its
# halo lists (2048 ids per 256 particles) and two 16-bit halo indices per
# slot.  Used for admission.
FOOTPRINT = {native.PD_FP64: (215.0, 4.0 + 48.0 + 4.0), native.PD_MIXED: (230.0 + 34.0, 4.0 + 4.0 + 4.0 + 4.0)}


@dataclass
class Request:
    rid: int
    arrival: float
    nx: int
    ny: int
    steps: int
    seed: int
    material: plates.Material
    v_load: float
    crack: tuple

    @property
    def particles(self):
        return self.nx * self.ny

    def plate(self):
        return plates.make_plate(self.nx, self.ny, seed=self.seed, crack=self.crack, material=self.material,
                                 v_load=self.v_load, steps=self.steps, name=f"req{self.rid}")


@dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    finished: float
    particles: int
    bonds: int
    steps: int
    digest: str
    broken: int
    state: tuple | None = None  # (u, bond mask) when the request id is in Server.keep

    @property
    def latency(self):
        return self.finished - self.arrival


def footprint(n, precision, bonds_per_particle=28.0):
    per_p, per_slot = FOOTPRINT[precision]
    return n * (per_p + per_slot * bonds_per_particle)


def make_requests(count, seed=0, lo=1e4, hi=2e6, steps_lo=200, steps_hi=2000, rate=None, load_work=None):
    """Seeded request stream: particle counts log-uniform in [lo, hi], square or
    2:1 plates, random crack (0.1-0.5 width, +-30 deg) and material as the
    batched workload, steps uniform in [steps_lo, steps_hi].  Arrivals are a
    Poisson process of `rate` requests/s (or back to back if rate is None)."""
    r = plates.uniform(seed, 21, np.arange(12 * count)).reshape(count, 12)
    reqs, t = [], 0.0
    for k in range(count):
        n = math.exp(math.log(lo) + (math.log(hi) - math.log(lo)) * r[k, 0])
        if r[k, 1] < 0.5:
            nx = ny = max(8, int(round(math.sqrt(n))))
        else:
            ny = max(8, int(round(math.sqrt(n / 2.0))))
            nx = 2 * ny
        steps = int(steps_lo + (steps_hi - steps_lo) * r[k, 2])
        mat = plates.Material(E=50e9 + 50e9 * r[k, 3], nu=0.2 + 0.15 * r[k, 4], rho=2440.0, s_c=5e-4)
        dx = 1e-3
        x0, y0 = -math.floor(nx / 2) * dx, -math.floor(ny / 2) * dx
        w, h = (nx - 1) * dx, (ny - 1) * dx
        crack = (x0 + (0.3 + 0.4 * r[k, 5]) * w, y0 + (0.3 + 0.4 * r[k, 6]) * h, (0.1 + 0.4 * r[k, 7]) * w,
                 math.radians(-30.0 + 60.0 * r[k, 8]))
        if rate:
            t += -math.log(max(1e-300, 1.0 - r[k, 9])) / rate
        reqs.append(Request(k, t, nx, ny, steps, seed * 100003 + k, mat, 0.5 + 1.5 * r[k, 10], crack))
    return reqs


def state_digest(ctx):
    u, v, _ = ctx.state()
    m = ctx.bond_mask()
    h = hashlib.sha256()
    for a in (u, v, m):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest(), int((m == 0).sum())


@dataclass
class _Parked:
    """A preempted request: its plate and its checkpoint (pd_checkpoint_save) in host memory."""
    request: Request
    plate: plates.Plate
    blob: bytes
    remaining: int
    admitted: float

    @property
    def rid(self):
        return self.request.rid

    @property
    def particles(self):
        return self.request.particles


@dataclass
class Server:
    """preempt: when the request at the head of the queue does not fit the HBM
    budget, active requests with at least `preempt_ratio` times its remaining
    work are checkpointed to host memory (largest first), freed, and queued
    again behind it; they resume from the checkpoint bit for bit."""
    precision: int = native.PD_MIXED
    device: int = 0
    budget_bytes: float = 150e9
    max_plates: int = 256
    chunk: int = 50
    batch_config: dict | None = None
    workers: int = 4
    builder_threads: int = 3  # device contexts built ahead of admission
    reader_threads: int = 2  # finished requests' results read (and their memory freed) off the loop
    preempt: bool = True
    preempt_ratio: float = 4.0
    keep: set = field(default_factory=set)  # request ids whose final (u, mask) the results keep
    results: list = field(default_factory=list)
    preemptions: int = 0

    def run(self, requests, stop_after=None):
        """Serve `requests` (arrival times relative to the start); returns metrics."""
        batch = native.Batch(precision=self.precision, device=self.device)
        if self.batch_config:
            batch.set_config(**self.batch_config)
        pending = deque(sorted(requests, key=lambda q: q.arrival))
        queue, active, used = deque(), {}, 0.0
        pool = ThreadPoolExecutor(max_workers=self.workers)  # host plates
        builders = ThreadPoolExecutor(max_workers=self.builder_threads)  # built while the GPU steps the batch
        readers = ThreadPoolExecutor(max_workers=self.reader_threads)  # results read while the loop goes on
        futs, building, reserved = {}, {}, 0.0
        t0 = time.perf_counter()
        busy = 0.0
        bond_steps = 0
        done = 0

        def build(q, plate_future):
            p = plate_future.result()
            return p, p.context(precision=self.precision, device=self.device)

        def start_build(q, need):
            nonlocal reserved
            building[q.rid] = (builders.submit(build, q, futs.pop(q.rid)), need)
            reserved += need

        # finished requests: their results are read (and their memory freed) on reader threads
        # while the loop admits and steps; `used` drops when a read completes (harvest)
        retired, reading = [], []

        def read(q, ctx, admitted, fin):
            dig, broken = state_digest(ctx)
            kept = (ctx.state()[0], ctx.bond_mask()) if q.rid in self.keep else None
            res = Result(q.rid, q.arrival, admitted, fin, q.particles, ctx.nnz, q.steps, dig, broken, kept)
            ctx.close()
            return res

        def harvest(wait=False):
            nonlocal used
            keep = []
            for fut, need in reading:
                if wait or fut.done():
                    self.results.append(fut.result())
                    used -= need
                else:
                    keep.append((fut, need))
            reading[:] = keep

        def finish():
            for q, ctx, admitted, fin, need in retired:
                reading.append((readers.submit(read, q, ctx, admitted, fin), need))
            retired.clear()

        while pending or queue or active:
            harvest()
            now = time.perf_counter() - t0
            while pending and pending[0].arrival <= now:
                q = pending.popleft()
                queue.append(q)
                if q.rid not in futs:
                    futs[q.rid] = pool.submit(q.plate)
            # prefetch the next arrivals' host plates too
            for q in list(pending)[: self.workers]:
                if q.rid not in futs:
                    futs[q.rid] = pool.submit(q.plate)
            # build the device contexts of arrived requests ahead of admission, in FIFO order,
            # while their footprint fits next to the active and building ones.  The requests
            # being built stay a prefix of the queue (a parked request, restored at its
            # admission, stops the scan), so their reserved memory never blocks the head.
            for q in list(queue)[: self.workers]:
                if isinstance(q, _Parked):
                    break
                if q.rid in building:
                    continue
                need = footprint(q.particles, self.precision)
                if used + reserved + need > self.budget_bytes or len(active) + len(building) >= self.max_plates:
                    break
                start_build(q, need)
            # admission: FIFO, by footprint and slots (preempting long requests if enabled)
            while queue and len(active) < self.max_plates:
                q = queue[0]
                need = footprint(q.particles, self.precision)
                if q.rid not in building:
                    if used + reserved + need > self.budget_bytes and active and self.preempt and \
                            not isinstance(q, _Parked):
                        freed, parked = self._preempt_for(q, need, used + reserved, active, batch)
                        used -= freed
                        at = 1  # behind the head and the requests already being built
                        while at < len(queue) and not isinstance(queue[at], _Parked) and queue[at].rid in building:
                            at += 1
                        for pk in reversed(parked):
                            queue.insert(at, pk)
                    # (a retired request still holds its memory until its results are read)
                    if used + reserved + need > self.budget_bytes and (active or building or retired or reading):
                        break
                if isinstance(q, _Parked):
                    queue.popleft()
                    ctx = q.plate.context(precision=self.precision, device=self.device)
                    ctx.restore(q.blob)
                    batch.add(ctx)
                    used += need
                    active[q.rid] = [q.request, ctx, q.remaining, q.admitted, need, q.plate]
                    continue
                if q.rid not in building:
                    start_build(q, need)
                fut, need = building[q.rid]
                if not fut.done() and active:
                    break  # keep the GPU busy; admit when its context is built
                p, ctx = fut.result()
                del building[q.rid]
                reserved -= need
                queue.popleft()
                batch.add(ctx)
                used += need
                active[q.rid] = [q, ctx, q.steps, time.perf_counter() - t0, need, p]
            if not active:
                finish()
                if reading and used + reserved > 0 and queue:
                    harvest(wait=True)  # the head may be waiting for memory that a read frees
                    continue
                if pending:
                    time.sleep(max(0.0, min(0.01, pending[0].arrival - (time.perf_counter() - t0))))
                continue
            k = min(self.chunk, min(a[2] for a in active.values()))
            batch.step(k)
            finish()  # the previous chunk's finished requests, while this chunk runs
            batch.synchronize()
            busy += batch.last_step_ms() / 1e3
            fin = time.perf_counter() - t0
            for rid in list(active):
                a = active[rid]
                a[2] -= k
                bond_steps += a[1].nnz * k
                if a[2] == 0:
                    batch.remove(a[1])
                    retired.append((a[0], a[1], a[3], fin, a[4]))
                    del active[rid]
                    done += 1
            if stop_after and done >= stop_after:
                break
        finish()
        harvest(wait=True)
        makespan = time.perf_counter() - t0
        readers.shutdown()
        pool.shutdown()
        for fut, _ in building.values():  # stopped early: contexts built ahead of admission
            fut.result()[1].close()
        builders.shutdown()
        batch.close()
        lat = np.array([r.latency for r in self.results])
        wait = np.array([r.admitted - r.arrival for r in self.results])
        arr = np.array([r.arrival for r in self.results])
        pct = (lambda a, q: float(np.percentile(a, q)) if a.size else None)
        return {
            "requests": len(self.results),
            "latency_samples": int(lat.size),
            "precision": "fp64" if self.precision == native.PD_FP64 else "mixed",
            "p50_latency_s": pct(lat, 50),
            "p95_latency_s": pct(lat, 95),
            "p99_latency_s": pct(lat, 99),
            "max_latency_s": float(lat.max()) if lat.size else None,
            "mean_latency_s": float(lat.mean()) if lat.size else None,
            "p50_queue_s": pct(wait, 50),
            "p99_queue_s": pct(wait, 99),
            "arrival_window_s": float(arr.max() - arr.min()) if arr.size else None,
            "makespan_s": makespan,
            "gpu_busy_frac": busy / makespan if makespan > 0 else None,
            "bond_updates_per_s": bond_steps / makespan if makespan > 0 else None,
            "bond_updates": bond_steps,
            "preemptions": self.preemptions,
        }

    def _preempt_for(self, q, need, used, active, batch):
        """Checkpoints and frees active requests (largest remaining work first,
        each with >= preempt_ratio x q's work) until q fits.  Returns the bytes
        freed and the parked requests (the caller queues them behind q)."""
        work_q = q.steps * q.particles
        victims = sorted(active.items(), key=lambda kv: -kv[1][2] * kv[1][0].particles)
        freed, parked = 0.0, []
        for rid, a in victims:
            if used - freed + need <= self.budget_bytes:
                break
            if a[2] * a[0].particles < self.preempt_ratio * work_q:
                break
            batch.remove(a[1])
            blob = a[1].checkpoint()
            a[1].close()
            parked.append(_Parked(a[0], a[5], blob, a[2], a[3]))
            freed += a[4]
            del active[rid]
            self.preemptions += 1
        return freed, parked


def solo_digest(request, precision, device=0):
    """The same request run alone (its own context, pd_step)."""
    ctx = request.plate().context(precision=precision, device=device)
    ctx.step(request.steps)
    d = state_digest(ctx)
    ctx.close()
    return d
