"""The N > 1 launch path on CPU (gloo, world size 2): bench.py's host-side
barrier / max / sum over ranks, per-rank replica workloads, and the
reference arm under torch.distributed.run (rank 0 runs and prints, the
other ranks exit 0).  The plate step does not shard: N GPUs run N replicas."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

SCRIPT = r"""
import json, sys
sys.path.insert(0, {root!r})
import bench
c = bench.Comm()
c.barrier()
out = {{"rank": c.rank, "world": c.world, "max": c.max(c.rank + 1.5), "sum": c.sum(c.rank + 1)}}
import importlib
pdg = importlib.import_module("2d_pd_gpu_gb300")
p = bench.replica_plate(pdg, 40, 0, c.rank)
out["seed_x0"] = float(p.x[0, 0])
out["n"] = int(p.n)
c.barrier()
c.close()
print(json.dumps(out))
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_comm_gloo_two_ranks():
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", SCRIPT.format(root=ROOT)], cwd=ROOT, env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=240)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    outs.sort(key=lambda d: d["rank"])
    for d in outs:
        assert d["world"] == 2 and d["max"] == 2.5 and d["sum"] == 3.0
    # weak scaling: every rank steps a plate of the same size from its own seed
    assert outs[0]["n"] == outs[1]["n"] and outs[0]["seed_x0"] != outs[1]["seed_x0"]


def test_reference_arm_under_torchrun():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference", "--gpus", "2", "--side", "60",
           "--steps", "2", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def test_gpus_flag_starts_the_ranks_itself():
    """`bench.py --gpus 2` with no launcher relaunches itself under
    torch.distributed.run: two ranks join (n_gpus counts the ranks in the
    process group), rank 0 alone prints; the config dict is the shared one."""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--side", "60", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env={k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and "rank 0 of 2" in d["parallelism"]
    sys.path.insert(0, ROOT)
    import argparse

    import bench

    want = bench.workload_config(argparse.Namespace(side=60), d["config"]["particles"], d["config"]["bonds"])
    assert d["config"] == want


def test_gpus_flag_must_match_the_launcher():
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--side", "40"], cwd=ROOT,
                       capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode != 0 and "WORLD_SIZE=1" in r.stderr
