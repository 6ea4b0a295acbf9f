"""Throughput of the explicit NOSB step on GB300 (bond-updates/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (N=1): the 1000 x 1000 FP64 plate -- 1,000,000 particles, ~27.9M
directed bonds, seeded +-0.01 dx jitter, a pre-crack of seeded length in
[0.2, 0.5] width at a seeded height, E=72 GPa, nu=0.33, rho=2440 kg/m^3,
s_c=5e-4 (bond breaking on), top/bottom 3 rows at +-1 m/s, dt = 0.8 CFL.
One bench step = one time step of the whole plate (drift, pass A, pass B).
Synthetic data (there is no public dataset for this path).  The state
(~2 GB of per-particle and per-bond arrays) is far larger than the 129 MB L2,
so no flush is needed between steps.

Reported: value = bond-updates/s over the timed K steps (CUDA events on the
context's stream, one graph of K steps); roofline of the dominant kernel
(per-kernel CUDA events over a second K-step pass); e2e = the same metric
through the public API with pinned host buffers (state uploaded before and
downloaded after every step); cpu_baseline = the oracle's C restatement
(OpenMP, all host cores) on a bounded sample of the same plate.  With
--impl reference, the reference arm: that CPU restatement alone.

Multi-GPU: independent replicas (the step is not sharded), one per rank,
launched by torch.distributed.run; value aggregates all ranks over the max
rank time.
"""
from __future__ import annotations

import argparse
import contextlib
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED_FP64_DFMA_PER_S = 6.27e11  # FP64 FMA rate of this GB300 (profiles/fp64_fma_rate_probe.txt), if the live probe fails


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# (start, end) of every timed region, perf_counter seconds: the clock record is taken over these
TIMED_WINDOWS = []


@contextlib.contextmanager
def timed():
    t0 = time.perf_counter()
    try:
        yield
    finally:
        TIMED_WINDOWS.append((t0, time.perf_counter()))


class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons while the run goes on; the
    record covers the samples taken inside timed regions (every sample if none fell in one)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append((time.perf_counter(), parts))

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        inside = [r for t, r in self.rows if any(a <= t <= b for a, b in TIMED_WINDOWS)]
        rows = inside if inside else [r for _, r in self.rows]
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows), "samples_whole_run": len(self.rows),
                "over": "timed regions" if inside else "whole run"}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Comm:
    """Host-side barrier / max over ranks (gloo); a no-op at N=1."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v):
        if not self.dist:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if not self.dist:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def byte_model(precision, n, nb):
    """Algorithmic bytes per launch (each array once per pass that must touch it)."""
    if precision == "fp64":
        return {"pass_a": 88.0 * n + 6.0 * nb, "pass_b": 160.0 * n + 5.0 * nb, "drift": 64.0 * n,
                "step": 248.0 * n + 11.0 * nb}
    return {"pass_a": 56.0 * n + 6.0 * nb, "pass_b": 92.0 * n + 5.0 * nb, "drift": 40.0 * n,
            "step": 148.0 * n + 11.0 * nb}


# DRAM bytes (read + write) per launch per bond, from one ncu capture of each
# pass on the 600 x 600 plate (10,031,592 bonds; profiles/passes_fp64_plate600.txt
# and profiles/passes_mixed_plate600.txt), scaled to a launch by its bonds:
# traffic grows with the bonds (and the particles, in the same proportion on
# these plates).
DRAM_BYTES_PER_BOND = {"fp64": {"pass_a": 265.71e6 / 10031592, "pass_b": 245.49e6 / 10031592},
                       "mixed": {"pass_a": 41.67e6 / 10031592, "pass_b": 55.35e6 / 10031592}}


def fp64_ops(n, nb):
    """FP64 operations per step of the FP64 form: pass A 8 per bond (d 2, D 4,
    penalty sum 2; the stretch test is certified in FP32 for nearly all bonds)
    + ~40 per particle, pass B 4 per bond + ~35 per particle."""
    return 12.0 * nb + 75.0 * n


def cpu_step_rate(plate, steps, nthreads, s_c=None):
    import pd_oracle as po

    rp, col = po.build_families(plate.x, plate.cutoff, plate.cracks, nthreads=nthreads)
    sim = po.OracleSim(plate.x, plate.vol, rp, col, E=plate.material.E, nu=plate.material.nu,
                       rho=plate.material.rho, dt=plate.dt, s_c=plate.material.s_c if s_c is None else s_c,
                       k_hg=plate.k_hg, damage_fail=plate.damage_fail, bc=plate.group_of,
                       group_kind=plate.group_kind, group_val=plate.group_val, nthreads=nthreads)
    sim.step(1)  # first touch
    t0 = time.perf_counter()
    sim.step(steps)
    dt = time.perf_counter() - t0
    return int(rp[-1]), dt


def replica_plate(pdg, side, seed, rank):
    """The plate rank `rank` steps: the same size on every rank (weak scaling),
    its own seed (jitter and crack), so replicas are independent solves."""
    return pdg.plates.config_plate_scale(side=side, seed=seed + rank)


def run_reference(args, comm):
    """Reference arm: the oracle's C restatement of the reference step, all host cores."""
    if comm.rank != 0:
        return
    pdg = importlib.import_module("2d_pd_gpu_gb300")
    plate = pdg.plates.config_plate_scale(side=args.side, seed=args.seed)
    nth = os.cpu_count() or 1
    import pd_oracle as po

    rp, col = po.build_families(plate.x, plate.cutoff, plate.cracks, nthreads=nth)
    sim = po.OracleSim(plate.x, plate.vol, rp, col, E=plate.material.E, nu=plate.material.nu,
                       rho=plate.material.rho, dt=plate.dt, s_c=plate.material.s_c, k_hg=plate.k_hg,
                       damage_fail=plate.damage_fail, bc=plate.group_of, group_kind=plate.group_kind, group_val=plate.group_val, nthreads=nth)
    nb = int(rp[-1])
    sim.step(max(args.warmup, 1))
    t0 = time.perf_counter()
    sim.step(args.steps)
    secs = time.perf_counter() - t0
    v = nb * args.steps / secs
    sample = f"{args.steps} full steps of the {args.side}x{args.side} FP64 plate ({nb} bonds), {nth} threads"
    print(json.dumps({
        "impl": "reference", "metric": "bond-updates/s", "value": v, "unit": "bond-updates/s", "n_gpus": comm.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, plate.n, nb),
        "parallelism": f"{nth} host threads on rank 0 of {comm.world}",
        "cpu_baseline": {"value": v, "unit": "bond-updates/s", "cores": nth, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "bond-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def workload_config(args, particles, bonds):
    """The workload both arms measure (identical dicts in both JSON lines)."""
    return {"workload": f"plate{args.side}x{args.side}-fp64-crack-sc5e-4", "particles": particles, "bonds": bonds,
            "precision": "fp64", "l2": "inputs larger than L2 (~2 GB state vs 129 MB L2), no flush"}


def measure(ctx, prec, args, comm, sampler=None):
    """Warm up, time K steps (one graph), then time every kernel of K more steps."""
    n, nb = ctx.n, ctx.nnz
    ctx.step(args.warmup)
    ctx.synchronize()
    comm.barrier()
    with timed():
        ms = ctx.step_timed(args.steps)
    comm.barrier()
    ms_max = comm.max(ms)
    value = comm.sum(nb * args.steps) / (ms_max / 1e3)
    prof = ctx.profile_steps(args.steps)
    model = byte_model(prec, n, nb)
    tot = sum(v[0] for v in prof.values())
    dom = max(("pass_a", "pass_b"), key=lambda k: prof[k][0])
    avg_ms = prof[dom][0] / max(prof[dom][1], 1)
    peaks, peak_kind = load_peaks()
    achieved = model[dom] / (avg_ms / 1e3) / 1e9
    kernels = {k: {"launches": prof[k][1], "avg_ms": prof[k][0] / max(prof[k][1], 1),
                   "share": prof[k][0] / tot if tot else None,
                   "achieved_gbs": (model[k] / (prof[k][0] / max(prof[k][1], 1) / 1e3) / 1e9) if prof[k][1] else None,
                   "algorithmic_bytes": model[k]}
               for k in prof}
    traffic = DRAM_BYTES_PER_BOND[prec][dom] * nb
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / peaks["hbm_gbs"], "traffic": traffic, "traffic_unit": "bytes per launch",
            # the DRAM bytes the kernel really moves (ncu), over the same live duration
            "frac_measured_traffic": traffic / (avg_ms / 1e3) / 1e9 / peaks["hbm_gbs"],
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum on the 600 x 600 plate, scaled by bonds",
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)", "algorithmic_bytes_per_launch": model[dom]}
    return value, ms_max / args.steps, kernels, roof


def accuracy(pdg, plate, device, checkpoints=(100, 500, 1000)):
    """Mixed vs FP64 from the same initial state: max / RMS displacement error
    (normwise), velocity error, and bond-mask mismatches at each checkpoint."""
    nat = pdg.native
    a = plate.context(precision=nat.PD_FP64, device=device)
    b = plate.context(precision=nat.PD_MIXED, device=device)
    out, done = {}, 0
    for t in checkpoints:
        a.step(t - done)
        b.step(t - done)
        done = t
        ua, va, _ = a.state()
        ub, vb, _ = b.state()
        ma, mb = a.bond_mask(), b.bond_mask()
        out[str(t)] = {"u_max_rel": float(np.abs(ub - ua).max() / np.abs(ua).max()),
                       "u_rms_rel": float(np.sqrt(((ub - ua) ** 2).mean() / (ua ** 2).mean())),
                       "v_max_rel": float(np.abs(vb - va).max() / np.abs(va).max()),
                       "mask_mismatch": int((ma != mb).sum()), "bonds_broken_fp64": int((ma == 0).sum())}
    a.close()
    b.close()
    return out


def e2e_leg(ctx, nat, comm, esteps, device, dropin=False):
    """The step end to end through the public API: pd_step_host(1) with the
    state in page-locked host buffers every step (read and written over the
    CPU-GPU link inside the timed region), and the same through the
    three-call sequence pd_set_state -> pd_step(1) -> pd_get_state.  dropin
    (FP64 contexts): also pd_compute_velocity, the reference GPU wrapper's
    one-call contract, on page-locked buffers (it changes the context's state:
    run it last)."""
    n, nb = ctx.n, ctx.nnz
    bufs = [nat.PinnedArray((n, 2)) for _ in range(3)]
    u, v, f = (b.array for b in bufs)
    u[:], v[:], f[:] = ctx.state()
    ctx.step_host(1, u, v, f)  # plans the pipeline (once per context), outside the timed region
    comm.barrier()
    with timed():
        t0 = time.perf_counter()
        for _ in range(esteps):
            ctx.step_host(1, u, v, f)
        secs = comm.max(time.perf_counter() - t0)
    out = {"value": comm.sum(nb * esteps) / secs, "unit": "bond-updates/s", "ms_per_step": 1e3 * secs / esteps,
           "h2d_bytes_per_step": 3 * 16 * n, "d2h_bytes_per_step": 3 * 16 * n, "steps": esteps,
           "api": "pd_step_host(1): u, v, f (FP64) copied in from page-locked host buffers slab by slab under "
                  "the first pass, and written back to them by each slab's last pass, every step"}
    comm.barrier()
    t0 = time.perf_counter()
    for _ in range(esteps):
        ctx._ck(nat.lib().pd_set_state(ctx.handle, nat.ptr(u), nat.ptr(v), nat.ptr(f)))
        ctx._ck(nat.lib().pd_step(ctx.handle, 1))
        ctx._ck(nat.lib().pd_get_state(ctx.handle, nat.ptr(u), nat.ptr(v), nat.ptr(f)))
    secs = comm.max(time.perf_counter() - t0)
    out["copies_api"] = {"value": comm.sum(nb * esteps) / secs, "api": "pd_set_state -> pd_step(1) -> pd_get_state"}
    for b in bufs:
        b.free()
    if dropin:
        bufs = [nat.PinnedArray((n, 2)) for _ in range(4)]
        u, v, a, f = (b.array for b in bufs)
        u[:], v[:], _ = ctx.state()
        a[:] = 0.0
        ctx.compute_velocity(u, v, a, netf=f)  # outside the timed region
        comm.barrier()
        t0 = time.perf_counter()
        for _ in range(esteps):
            ctx.compute_velocity(u, v, a, netf=f)
        secs = comm.max(time.perf_counter() - t0)
        out["dropin_api"] = {"value": comm.sum(nb * esteps) / secs, "unit": "bond-updates/s",
                             "ms_per_step": 1e3 * secs / esteps, "h2d_bytes_per_step": 3 * 16 * n,
                             "d2h_bytes_per_step": 3 * 16 * n, "steps": esteps,
                             "api": "pd_compute_velocity (compute_velocity_GPU_host's contract, one force + kick "
                                    "per call): u, velocity, acce in from page-locked buffers, velocity, acce, "
                                    "netF back, by the same slab pipeline"}
        for b in bufs:
            b.free()
    # the link bound: the step's bytes each way at the measured concurrent copy rate
    h2d, d2h, both = nat.probe_link_rates(3 * 16 * n, device)
    out["link"] = {"h2d_gbs": h2d, "d2h_gbs": d2h, "both_gbs_per_direction": both,
                   "bound_ms_per_step": 3 * 16 * n / (both * 1e9) * 1e3,
                   "source": "pd_probe_link_rates: copy engines, page-locked buffers of the step's size"}
    return out


# The reference's only published timings: one call of its velocity step on the
# Hassa mesh (4,064 particles, 107,996 bonds) with its default bond-associated
# weights n1 = n2 = 10 -- output/cpu_output.txt:9 (sequential computeVelocity)
# and output/gpu_output.txt:9 (compute_velocity_GPU_host, including its
# per-call cudaMalloc / copies / free; that kernel's results are wrong,
# include/mechanics.cuh:165 uses the initial instead of the current position).
REFERENCE_HASSA_CPU_S = 69.967052
REFERENCE_HASSA_GPU_S = 0.609138


def run_bond_assoc(pdg, calls=6):
    """The reference's published problem through the drop-in: the Hassa mesh,
    n1 = n2 = 10, the reference GPU main's call sequence, compute_velocity_GPU_host
    timed per call with host buffers (as the reference times it), and the same
    step device-resident (pd_step_timed)."""
    import tempfile

    exe = os.path.join(os.path.dirname(pdg.native.LIB_PATH), "pd_hassa_timing")
    with tempfile.TemporaryDirectory() as td:
        open(os.path.join(td, "2D_Hassa_test_mesh.dat"), "w").write(pdg.plates.hassa_mesh_text())
        r = subprocess.run([exe, "10", "10", str(calls)], cwd=td, capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        return {"error": r.stderr[-500:]}
    d = json.loads(r.stdout.strip().splitlines()[-1])
    nb = d["bonds"]
    call_s = d["median_call_s"]
    dev_s = d["device_step_ms_median"] / 1e3
    return {"workload": "hassa-mesh-4064-bond-associated-n1=n2=10", "particles": d["particles"], "bonds": nb,
            "e2e": {"value": nb / call_s, "unit": "bond-updates/s", "seconds_per_call": call_s,
                    "first_call_s": d["first_call_s"], "calls": d["calls"],
                    "api": "compute_velocity_GPU_host (C++ drop-in, host vectors in and out every call)"},
            "device": {"value": nb / dev_s, "unit": "bond-updates/s", "ms_per_step": d["device_step_ms_median"],
                       "api": "pd_step_timed(1), CUDA events"},
            "reference_published": {"cpu_s": REFERENCE_HASSA_CPU_S, "gpu_s": REFERENCE_HASSA_GPU_S,
                                    "gpu_parity": "not parity-correct (wrong results, up to 78% off the CPU path)",
                                    "source": "output/cpu_output.txt:9, output/gpu_output.txt:9"},
            "speedup_e2e_vs_reference_cpu": REFERENCE_HASSA_CPU_S / call_s,
            "speedup_e2e_vs_reference_gpu": REFERENCE_HASSA_GPU_S / call_s,
            "speedup_first_call_vs_reference_gpu": REFERENCE_HASSA_GPU_S / d["first_call_s"]}


def run_mixed_scale(args, pdg, device, comm):
    """The mixed form on a scale_side x scale_side plate (16M particles at 4000):
    how the bandwidth-class path holds up when nothing of the state fits L2."""
    t0 = time.perf_counter()
    plate = pdg.plates.config_plate_scale(side=args.scale_side, seed=args.seed)
    ctx = plate.context(precision=pdg.native.PD_MIXED, device=device)
    setup_s = time.perf_counter() - t0
    sub = argparse.Namespace(**vars(args))
    sub.steps = min(args.steps, 20)
    value, step_ms, kernels, roof = measure(ctx, "mixed", sub, comm)
    out = {"value": value, "unit": "bond-updates/s", "ms_per_step": step_ms, "steps": sub.steps,
           "particles": plate.n, "bonds": ctx.nnz, "setup_s": setup_s, "roofline": roof, "kernels": kernels,
           "workload": f"plate{args.scale_side}x{args.scale_side}-mixed-crack-sc5e-4"}
    ctx.close()
    return out


def run_batch(args, pdg, device):
    """Ragged batch: 256 plates, side U[50,400], seeded crack / material / load,
    stepped together by pd_batch with the autotuned launch shape."""
    nat = pdg.native
    at = importlib.import_module("2d_pd_gpu_gb300.autotune")
    specs = pdg.plates.batch_plate_specs(args.batch_plates, seed=args.seed)
    out = {}
    for name, prec in (("fp64", nat.PD_FP64), ("mixed", nat.PD_MIXED)):
        t0 = time.perf_counter()
        ctxs = [pdg.plates.plate_from_spec(s, steps=500).context(precision=prec, device=device) for s in specs]
        setup = time.perf_counter() - t0
        b = nat.Batch(precision=prec, device=device)
        for c in ctxs:
            b.add(c)
        info = b.info()
        best, timings = at.tune_batch(b, steps=3, warmup=1)
        for c in ctxs:
            c.reset()
        b.step(args.warmup)
        b.synchronize()
        with timed():
            ms = b.step_timed(args.batch_steps)
        val = info["bonds"] * args.batch_steps / (ms / 1e3)
        model = byte_model(name, info["particles"], info["bonds"])["step"]
        peaks, _ = load_peaks()
        ach = model / (ms / args.batch_steps / 1e3) / 1e9
        out[name] = {"value": val, "unit": "bond-updates/s", "ms_per_step": ms / args.batch_steps,
                     "plates": info["plates"], "particles": info["particles"], "bonds": info["bonds"],
                     "steps": args.batch_steps, "setup_s": setup, "config": best,
                     "mode": {0: "graph of phase kernels", 1: "persistent cooperative kernel",
                              2: "every plate's own step graph, concurrently"}[best["persistent"]],
                     "candidates_ms": {k: round(v, 4) for k, v in sorted(timings.items(), key=lambda kv: kv[1])[:6]},
                     "achieved_gbs_step_model": ach, "frac_hbm": ach / peaks["hbm_gbs"],
                     "gpu_launches": {0: 1 + 2 * args.batch_steps, 1: 1,
                                      2: info["plates"] * (1 + 2 * args.batch_steps)}[best["persistent"]]}
        b.close()
        for c in ctxs:
            c.close()
    return out


def run_serve(args, pdg, device, capacity, configs):
    """Served mixed workload: Poisson stream at ~80% of the measured batch
    capacity, particle counts log-uniform 10k-2M, steps U[200,2000], admission
    by HBM footprint under 150 GB, continuous batching."""
    nat = pdg.native
    serve = importlib.import_module("2d_pd_gpu_gb300.serve")
    out = {}
    fp64_count = args.serve_fp64_requests or max(4, args.serve_requests // 4)
    for name, prec, count in (("mixed", nat.PD_MIXED, args.serve_requests), ("fp64", nat.PD_FP64, fp64_count)):
        probe = serve.make_requests(count, seed=args.seed + 17)
        work = float(np.mean([27.9 * q.particles * q.steps for q in probe]))
        rate = args.serve_load * capacity[name] / work
        reqs = serve.make_requests(count, seed=args.seed + 17, rate=rate)
        # the mixed results' error against the FP64 form, on the three smallest requests
        sample = sorted(reqs, key=lambda q: q.particles * q.steps)[:3] if prec == nat.PD_MIXED else []
        srv = serve.Server(precision=prec, device=device, budget_bytes=150e9, chunk=args.serve_chunk,
                           batch_config=configs.get(name), keep={q.rid for q in sample})
        with timed():
            m = srv.run(reqs)
        # the load the stream actually offered: its bond updates over its arrival window, against capacity
        window = max(q.arrival for q in reqs) - min(q.arrival for q in reqs)
        offered = m["bond_updates"] / window / capacity[name] if window > 0 else None
        m.update({"arrival_rate_per_s": rate, "offered_load_target": args.serve_load,
                  "offered_load_achieved": offered, "capacity_bond_updates_per_s": capacity[name],
                  "particles_range": [min(q.particles for q in reqs), max(q.particles for q in reqs)]})
        if sample:
            by = {r.rid: r for r in srv.results}
            acc = []
            for q in sample:
                ref = q.plate().context(precision=nat.PD_FP64, device=device)
                ref.step(q.steps)
                u64, m64 = ref.state()[0], ref.bond_mask()
                ref.close()
                u32, m32 = by[q.rid].state
                du = np.abs(u32 - u64)
                acc.append({"rid": q.rid, "particles": q.particles, "steps": q.steps,
                            "u_max_rel": float(du.max() / np.abs(u64).max()),
                            "u_rms_rel": float(np.sqrt((du ** 2).mean() / (u64 ** 2).mean())),
                            "mask_mismatch": int((m32 != m64).sum()), "bonds_broken_fp64": int((m64 == 0).sum())})
            m["accuracy_vs_fp64"] = acc
        out[name] = m
    return out


def run_serve_only(args, comm):
    """The batch leg (capacity, autotuned launch shape) and the serve leg alone:
    long request streams whose percentiles need more time than the default run."""
    pdg = importlib.import_module("2d_pd_gpu_gb300")
    device = comm.local
    sampler = ClockSampler(device)
    sampler.start()
    result = {"metric": "served bond-updates/s and completion latency", "n_gpus": 1, "data": "synthetic",
              "config": {"workload": "serve: Poisson stream, plates 10k-2M particles log-uniform, 200-2000 steps, "
                                     "150 GB HBM budget"}}
    if comm.rank == 0:
        result["batch"] = run_batch(args, pdg, device)
        cap = {k: v["value"] for k, v in result["batch"].items()}
        cfgs = {k: v["config"] for k, v in result["batch"].items()}
        result["serve"] = run_serve(args, pdg, device, cap, cfgs)
    result["clocks"] = sampler.stop()
    if comm.rank == 0:
        print(json.dumps(result), flush=True)


def run_ours(args, comm):
    if args.serve_only:
        return run_serve_only(args, comm)
    pdg = importlib.import_module("2d_pd_gpu_gb300")
    nat = pdg.native
    plate = replica_plate(pdg, args.side, args.seed, comm.rank)
    device = comm.local
    sampler = ClockSampler(device)
    sampler.start()
    ctx = plate.context(precision=nat.PD_FP64, device=device)
    n, nb = ctx.n, ctx.nnz
    value, step_ms, kernels, roof = measure(ctx, "fp64", args, comm)
    result = {
        "metric": "bond-updates/s", "value": value, "unit": "bond-updates/s", "n_gpus": comm.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded plate generator)",
        "config": workload_config(args, n, nb),
        "parallelism": f"replicas x{comm.world} (one independent plate per GPU)",
        "gpu_launches": 1 + 2 * args.steps,
        "roofline": roof,
        "kernels": kernels,
    }
    ops = fp64_ops(n, nb) / (step_ms / 1e3)
    try:
        peak64, peak32 = nat.probe_fma_rates(device)
        src = "pd_probe_fma_rates on this GPU, measured in this run"
    except Exception:
        peak64, peak32, src = MEASURED_FP64_DFMA_PER_S, None, "recorded DFMA rate (profiles/fp64_fma_rate_probe.txt)"
    result["fp64_alu"] = {"ops_per_s": ops, "peak_ops_per_s": peak64, "frac": ops / peak64,
                          "ops_per_step": fp64_ops(n, nb), "peak_source": src, "fp32_fma_per_s": peak32}
    # the FP64 step's binding limit is the FP64 pipe, not HBM (ncu: FP64 pipe 83-87 % busy)
    result["roofline"]["binding"] = {"limit": "fp64_pipe", "frac": ops / peak64,
                                     "why": "GB300 executes FP64 at 1/58 of its FP32 rate; 12 FP64 operations "
                                            "per bond take ~8x longer than the step's algorithmic HBM bytes"}
    # end to end through the public API with pinned host buffers, every step
    if not args.no_e2e:
        result["e2e"] = e2e_leg(ctx, nat, comm, min(args.steps, args.e2e_steps), device, dropin=True)
    ctx.close()
    if not args.no_mixed:
        mctx = plate.context(precision=nat.PD_MIXED, device=device)
        mvalue, mstep_ms, mkernels, mroof = measure(mctx, "mixed", args, comm)
        result["mixed"] = {"value": mvalue, "unit": "bond-updates/s", "ms_per_step": mstep_ms,
                           "speedup_vs_fp64": mvalue / value, "dtype": "f32 bonds + f64 K^-1/det",
                           "roofline": mroof, "kernels": mkernels, "gpu_launches": 1 + 2 * args.steps}
        if not args.no_e2e:
            me2e = e2e_leg(mctx, nat, comm, min(args.steps, args.e2e_steps), device)
            me2e["speedup_vs_fp64_e2e"] = me2e["value"] / result["e2e"]["value"] if "e2e" in result else None
            result["mixed"]["e2e"] = me2e
        mctx.close()
        if not args.no_accuracy and comm.rank == 0:
            result["mixed"]["accuracy_vs_fp64"] = accuracy(pdg, plate, device)
        if args.scale_side > 0:
            result["mixed_scale"] = run_mixed_scale(args, pdg, device, comm)
    if comm.rank == 0 and not args.no_bond_assoc:
        result["bond_assoc"] = run_bond_assoc(pdg)
    if not args.no_batch and comm.rank == 0:
        result["batch"] = run_batch(args, pdg, device)
        if not args.no_serve:
            cap = {k: v["value"] for k, v in result["batch"].items()}
            cfgs = {k: v["config"] for k, v in result["batch"].items()}
            result["serve"] = run_serve(args, pdg, device, cap, cfgs)
    result["clocks"] = sampler.stop()
    if comm.rank == 0 and not args.no_cpu:
        nth = os.cpu_count() or 1
        nbc, secs = cpu_step_rate(plate, args.cpu_steps, nth)
        result["cpu_baseline"] = {"value": nbc * args.cpu_steps / secs, "unit": "bond-updates/s", "cores": nth,
                                  "kind": "port",
                                  "sample": f"{args.cpu_steps} steps of the same {args.side}x{args.side} plate "
                                            f"({nbc} bonds), oracle C restatement, OpenMP {nth} threads"}
    if comm.rank == 0:
        print(json.dumps(result), flush=True)


def relaunch(n):
    """--gpus N without a launcher: start N ranks (one per GPU) under
    torch.distributed.run on this node, rendezvous on 127.0.0.1; returns
    the launcher's exit status."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.run(cmd).returncode


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--side", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-bond-assoc", action="store_true")
    ap.add_argument("--scale-side", type=int, default=4000, help="mixed form on this plate too (0: skip)")
    ap.add_argument("--batch-plates", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=500)
    ap.add_argument("--serve-requests", type=int, default=64, help="mixed requests in the serve leg")
    ap.add_argument("--serve-fp64-requests", type=int, default=0, help="FP64 requests (0: a quarter of the mixed)")
    ap.add_argument("--serve-load", type=float, default=0.8, help="offered load, of the measured batch capacity")
    ap.add_argument("--serve-only", action="store_true",
                    help="only the batch leg (for the capacity) and the serve leg; prints their JSON line")
    ap.add_argument("--serve-chunk", type=int, default=50)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    launched = os.environ.get("WORLD_SIZE")
    if launched is None and args.gpus > 1:
        sys.exit(relaunch(args.gpus))
    if int(launched or 1) != args.gpus:
        sys.exit(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={launched}: launch one rank per GPU")
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    comm = Comm()
    try:
        if args.impl == "reference":
            run_reference(args, comm)
        else:
            run_ours(args, comm)
    finally:
        comm.close()


if __name__ == "__main__":
    main()
