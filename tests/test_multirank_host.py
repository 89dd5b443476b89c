"""Host logic of the multi-GPU paths, on CPU with the gloo backend (world size 2).

The single-chain sweep does not shard (replicas only); batched instances are
split across ranks with no data-path collective, and only the per-instance
results are gathered.  These tests cover that split with the library's own
(host-only) batched plans per rank and the aggregation of rank timings (max
over ranks) the benchmark uses."""
import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def test_shard_covers_every_instance_once():
    from syngular_gb300.batched import shard

    idx = list(range(37))
    for world in (1, 2, 3, 8):
        parts = [shard(idx, r, world) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == idx
        assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1


def _instances(count=9, seed=4):
    """Host-side shapes of uneven batched instances: (wshape, xshape, chi)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(3, 9))
        d = int(rng.choice([2, 3]))
        chi = int(rng.integers(2, 9))
        D = int(rng.choice([2, 4]))
        xb = [1] + [chi] * (n - 1) + [1]
        wb = [1] + [D] * (n - 1) + [1]
        xs = [v for k in range(n) for v in (xb[k], d, xb[k + 1])]
        ws = [v for k in range(n) for v in (wb[k], d, d, wb[k + 1])]
        out.append((ws, xs, int(rng.integers(2, 7))))
    return out


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from syngular_gb300 import _lib as L
    from syngular_gb300.batched import NativePlan, shard

    shapes = _instances()
    mine = shard(list(range(len(shapes))), rank, world)
    # this rank's own batched plan (host-only: sizes, lane deal, rounded shapes)
    plan = NativePlan([shapes[i] for i in mine], precision=L.PREC_BF16X6, lanes=2)
    local = {i: plan.out_shapes[j] for j, i in enumerate(mine)}
    gathered = [None] * world
    dist.all_gather_object(gathered, (rank, local, plan.ws_bytes))
    # max-over-ranks timing, as the benchmark reports it
    t = torch.tensor([1.0 + rank], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    q.put((rank, gathered, float(t.item())))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_gather_sharded_plans():
    """Each of two gloo ranks builds the library's batched plan for its own
    shard of the instances; the gathered rounded-core shapes cover every
    instance once and equal those of one plan over the whole batch."""
    import __graft_entry__ as g

    g.build()
    from syngular_gb300 import _lib as L
    from syngular_gb300.batched import NativePlan

    shapes = _instances()
    whole = NativePlan(shapes, precision=L.PREC_BF16X6, lanes=2)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, gathered, tmax in out:
        assert tmax == 2.0
        merged = {}
        for _r, local, ws in gathered:
            assert ws > 0
            assert not (set(local) & set(merged)), "an instance was planned on two ranks"
            merged.update(local)
        assert sorted(merged) == list(range(len(shapes)))
        for i in range(len(shapes)):
            assert [tuple(s) for s in merged[i]] == [tuple(s) for s in whole.out_shapes[i]]
