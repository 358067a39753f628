"""CPU, two ranks over gloo: the multi-GPU bench path is replicas only —
each rank predicts its own structures (disjoint seeds), the ranks meet at a
barrier around the timed region and the slowest rank's time is taken
(bench.py dist_setup / barrier / max_over_ranks / rank_seeds).  No GPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import json, os, sys, time
sys.path.insert(0, os.environ["FGB_ROOT"])
import bench
import torch.distributed as dist
rank, world, local = bench.dist_setup(0)
assert dist.get_backend() == "gloo" and world == 2
bench.barrier(world)
t = bench.max_over_ranks(1.5 + rank, world)
seeds = bench.rank_seeds(2100, rank, 4)
allseeds = [None] * world
dist.all_gather_object(allseeds, seeds)
bench.barrier(world)
if rank == 0:
    with open(os.environ["FGB_OUT"], "w") as f:
        json.dump({"max": t, "seeds": allseeds}, f)
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_gloo_replicas(tmp_path):
    pytest.importorskip("torch.distributed")
    script = tmp_path / "ranks.py"
    script.write_text(SCRIPT)
    out = tmp_path / "out.json"
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                   FGB_ROOT=ROOT, FGB_OUT=str(out), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env,
                                      stdout=subprocess.PIPE,
                                      stderr=subprocess.STDOUT))
    for p in procs:
        o, _ = p.communicate(timeout=120)
        assert p.returncode == 0, o.decode()[-2000:]
    res = json.loads(out.read_text())
    assert res["max"] == 2.5          # the slower rank's time
    s0, s1 = res["seeds"]
    assert len(s0) == len(s1) == 4 and not set(s0) & set(s1)


def test_reference_arm_two_ranks():
    """bench.py --impl reference under two gloo ranks: rank 0 alone times
    the CPU oracle and prints one JSON line; rank 1 exits 0 without work."""
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                   CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen(
            [sys.executable, os.path.join(ROOT, "bench.py"), "--impl",
             "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"],
            env=env, cwd=ROOT, stdout=subprocess.PIPE,
            stderr=subprocess.PIPE))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=600)
        assert p.returncode == 0, e.decode()[-2000:]
        outs.append([l for l in o.decode().splitlines() if l.startswith("{")])
    assert outs[1] == [] and len(outs[0]) == 1
    line = json.loads(outs[0][0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["unit"] == "atoms/s"
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"] == {"value": line["value"], "unit": "atoms/s",
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
