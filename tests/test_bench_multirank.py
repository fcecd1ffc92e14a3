"""The N > 1 path of bench.py on CPU: two gloo ranks combine their step
times with a max (the job ends with its slowest replica) and report the
whole-job rate; the reference arm prints only on rank 0."""

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys, json
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
dist.init_process_group("gloo")
r = dist.get_rank(); w = dist.get_world_size()
import bench
times = bench.slowest_rank([0.5 + r, 0.1 * (r + 1), 0.2], w)
rate = bench.job_rate(1e9, w, times[0])
dist.barrier()
print(json.dumps({"rank": r, "times": times, "rate": rate}))
dist.destroy_process_group()
"""


def _run_ranks(script, extra_env=None):
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2",
                   LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT="29533")
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, "-c", script, ROOT],
                                      env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err[-2000:]
        outs.append(out)
    return outs


def test_two_gloo_ranks_take_the_slowest_time():
    pytest.importorskip("torch")
    outs = _run_ranks(CHILD)
    res = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    for r in res:
        assert r["times"] == [1.5, 0.2, 0.2]
        assert abs(r["rate"] - 2 * 1e9 / 1.5 / 1e9) < 1e-12


def test_reference_arm_prints_on_rank_zero_only():
    pytest.importorskip("torch")
    script = r"""
import sys
sys.path.insert(0, sys.argv[1])
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
            "--n", "2048", "--cpu-ni", "64"]
import bench
bench.main()
"""
    outs = _run_ranks(script)
    lines = [[l for l in o.splitlines() if l.startswith("{")] for o in outs]
    assert len(lines[0]) == 1 and len(lines[1]) == 0
    rec = json.loads(lines[0][0])
    assert rec["impl"] == "reference" and rec["value"] > 0
    assert rec["e2e"]["h2d_bytes_per_step"] == 0
