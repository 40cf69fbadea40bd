"""The benchmark's multi-rank host logic (replicas only: no collective on the
data path) as two gloo ranks on the CPU: rendezvous, barrier, and the max of
the per-rank times that the whole-job throughput divides by."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, os, sys
sys.path.insert(0, {root!r})
import bench
ws, rank, local = bench.dist_init()
bench.barrier(ws)
t = bench.max_over_ranks(10.0 + 5.0 * rank, ws)   # per-rank "ms"
value = 1e12 * ws * 3 / (t / 1e3) / 1e12            # flops x ranks x steps / max time
import torch.distributed as dist
dist.destroy_process_group()
print(json.dumps({{"rank": rank, "ws": ws, "max_ms": t, "value": value}}))
"""


def test_two_gloo_ranks(tmp_path):
    script = tmp_path / "child.py"
    script.write_text(CHILD.format(root=ROOT))
    env = dict(os.environ, MGB_BENCH_BACKEND="gloo", MASTER_ADDR="127.0.0.1", MASTER_PORT="29571",
               WORLD_SIZE="2", CUDA_VISIBLE_DEVICES="")
    procs = []
    for r in range(2):
        e = dict(env, RANK=str(r), LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=e, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["ws"] == 2 and o["max_ms"] == 15.0
        assert abs(o["value"] - 2 * 3 / 0.015) < 1e-9
