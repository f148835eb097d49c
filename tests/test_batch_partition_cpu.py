"""CPU: the data-parallel split of a batch of independent GPs (each rank builds
a BatchPlan over its share; the only collective gathers the results), run as
two gloo ranks."""
import os

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from gpjax_gb300.objectives import gather_instance_results, partition_instances


def test_partition_balances_cubic_cost_and_covers_every_instance():
    rng = np.random.default_rng(0)
    ns = rng.integers(64, 2049, 512)
    for world in (1, 2, 3, 8):
        parts = partition_instances(ns, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(ns)))
        loads = [sum(float(ns[i]) ** 3 for i in p) for p in parts]
        # greedy largest-first: the spread is at most the largest single cost
        assert max(loads) - min(loads) <= float(ns.max()) ** 3
    assert partition_instances([5, 5], 4)[2:] == [[], []]


def _rank(rank, world, port, ns, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = partition_instances(ns, world)[rank]
        # stand-in for the plan's results: a value that identifies the instance
        mll = torch.tensor([1000.0 * i + ns[i] for i in mine], dtype=torch.float64)
        out = gather_instance_results(mll, mine, len(ns))
        q.put((rank, out.numpy().tolist()))
    finally:
        dist.destroy_process_group()


def test_gather_restores_the_original_order_over_two_gloo_ranks():
    ns = [100, 2000, 64, 1500, 900, 300, 1200]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, ns, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = [1000.0 * i + ns[i] for i in range(len(ns))]
    assert res[0] == want and res[1] == want
