"""Data-parallel collapsed ELBO, host side, as two gloo ranks on CPU:

* the row partition covers every row once;
* the exchange hook the library calls (objectives.allreduce_callback) sums a
  float64 region of a rank's workspace over the ranks at the byte offset the
  library names;
* the decomposition the sharded C path follows -- each rank's statistics of
  its rows (P = Kzx Kxz, c = Kzx d, d^T d, sum k(x, x), n), one sum over the
  ranks, then the replicated m x m algebra -- gives the single-rank ELBO of
  the whole dataset (objectives.py:341-416)."""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, os, sys
import numpy as np, torch, torch.distributed as dist
sys.path.insert(0, sys.argv[1])
from gpjax_gb300 import objectives
from oracle import gp_oracle as O
dist.init_process_group("gloo")
rank, world = dist.get_rank(), dist.get_world_size()
# the exchange hook on a CPU "workspace": rank r fills doubles with r + 1 at byte offset 512
ws = torch.zeros(4096, dtype=torch.uint8)
ws.narrow(0, 512, 8 * 10).view(torch.float64).fill_(rank + 1.0)
cb = objectives.allreduce_callback(ws)
status = cb(None, 512, 10, None)
summed = ws.narrow(0, 512, 80).view(torch.float64).tolist()
untouched = float(ws.narrow(0, 0, 512).view(torch.float64).abs().sum())
# the statistics decomposition on this rank's rows
rng = np.random.default_rng(3)
n, m, d = 1001, 24, 3
x = rng.standard_normal((n, d)); y = np.sin(x).sum(1, keepdims=True) + 0.1 * rng.standard_normal((n, 1))
z = x[rng.choice(n, m, replace=False)]
ls = np.array([0.7, 1.1, 1.6])
rows = objectives.shard_rows(n, world, rank)
st = O.sgpr_statistics(O.RBF, x[rows], y[rows], z, ls, 1.3, 0.1)
vec = torch.tensor(np.concatenate([st["P"].ravel(), st["c"], [st["dd"], st["kdiag"], st["n"]]]))
dist.all_reduce(vec)
v = vec.numpy()
tot = {"P": v[:m * m].reshape(m, m), "c": v[m * m:m * m + m], "dd": v[-3], "kdiag": v[-2],
       "n": int(round(v[-1]))}
elbo = O.collapsed_elbo_from_statistics(O.RBF, tot, z, ls, 1.3, 0.25)
full = O.collapsed_elbo(O.RBF, x, y, z, ls, 1.3, 0.25, 0.1)
print(json.dumps({"rank": rank, "status": status, "summed": summed, "untouched": untouched,
                  "rows": [rows.start, rows.stop], "elbo": elbo, "full": full}))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_rows_partition():
    from gpjax_gb300.objectives import shard_rows
    for n in (1, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            if world > n:
                continue
            seen = np.zeros(n, int)
            for r in range(world):
                sl = shard_rows(n, world, r)
                seen[sl] += 1
                assert sl.stop - sl.start in (n // world, n // world + 1)
            assert (seen == 1).all()
    with pytest.raises(ValueError):
        shard_rows(10, 2, 2)


def test_two_gloo_ranks_sum_statistics_to_the_full_elbo():
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT, ROOT], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=180)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    outs.sort(key=lambda o: o["rank"])
    assert outs[0]["rows"] == [0, 501] and outs[1]["rows"] == [501, 1001]
    for o in outs:
        assert o["status"] == 0
        assert o["summed"] == [3.0] * 10       # 1 + 2 over the two ranks
        assert o["untouched"] == 0.0           # nothing outside the named region
        assert o["elbo"] == pytest.approx(o["full"], rel=1e-11)
