"""The multi-GPU path of bench.py is replicas only (the Cholesky does not
shard): one process per GPU, a barrier, the max of the ranks' times and a
whole-job value of N x steps over it.  Here two gloo ranks run that host logic
on CPU, and a non-zero rank of the reference arm exits without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, sys, torch
sys.path.insert(0, sys.argv[1])
import bench
r = bench.Replicas("gloo")
r.barrier()
t = r.max(1.0 + 0.5 * r.rank, torch.device("cpu"))
print(json.dumps({"rank": r.rank, "world": r.world, "t": t, "value": r.value(10, t)}))
r.barrier()
r.close()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, world, port):
    env = dict(os.environ)
    env.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
               MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    return env


def test_replicas_two_gloo_ranks():
    port = _free_port()
    procs = [subprocess.Popen([sys.executable, "-c", RANK_SCRIPT, ROOT], env=_env(r, 2, port),
                              stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
             for r in range(2)]
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    outs.sort(key=lambda o: o["rank"])
    assert [o["rank"] for o in outs] == [0, 1]
    for o in outs:
        assert o["world"] == 2
        assert o["t"] == pytest.approx(1.5)        # the slowest rank's time
        assert o["value"] == pytest.approx(2 * 10 / 1.5)


def test_reference_arm_nonzero_rank_exits_quietly():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], env=_env(1, 2, _free_port()),
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_json_contract():
    """Rank 0 of the reference arm prints one JSON line with the keys the
    bench contract asks for (small workload: seconds of CPU)."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--n", "512", "--steps", "1", "--warmup", "0"], env=_env(0, 1, _free_port()),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert "n=512" in line["cpu_baseline"]["sample"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
