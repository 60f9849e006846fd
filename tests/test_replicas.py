"""The N > 1 bench path on CPU: replicas only (one field does not shard),
so ranks exchange nothing but the timing.  Two gloo ranks on 127.0.0.1
check the whole-job value (all ranks' grid-point steps over the slowest
rank's time), and the reference arm prints on rank 0 only."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, os.environ["VK_ROOT"])
import torch.distributed as dist
import bench
dist.init_process_group("gloo", init_method="env://")
rank = dist.get_rank()
value, ms_max = bench.replica_throughput(10.0 + 5.0 * rank, dist.get_world_size(), 64 * 64, 20, 3, dist, "cpu")
print(json.dumps({"rank": rank, "value": value, "ms_max": ms_max}))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replica_throughput_two_gloo_ranks():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), VK_ROOT=ROOT)
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    expect = 2 * 64 * 64 * 20 * 3 / 15e-3
    for o in outs:
        assert o["ms_max"] == 15.0
        assert abs(o["value"] - expect) <= 1e-9 * expect


def test_replica_throughput_single_rank_is_local():
    sys.path.insert(0, ROOT)
    import bench
    value, ms = bench.replica_throughput(4.0, 1, 100, 2, 5)
    assert ms == 4.0 and abs(value - 100 * 2 * 5 / 4e-3) < 1e-6


def _reference_arm(rank):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank))
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                           "--n", "64", "--steps", "2", "--warmup", "1"],
                          env=env, capture_output=True, text=True, timeout=300)


def test_reference_arm_prints_on_rank0_only():
    r1 = _reference_arm(1)
    assert r1.returncode == 0, r1.stderr
    assert r1.stdout.strip() == ""
    r0 = _reference_arm(0)
    assert r0.returncode == 0, r0.stderr
    lines = [l for l in r0.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
