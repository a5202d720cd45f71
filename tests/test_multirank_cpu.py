"""The multi-rank benchmark path on CPU: two gloo ranks (world size 2).

Each rank solves its own seeded snapshot (weak scaling, no data-path
collective); the job's step time is the maximum over ranks; only rank 0 of
the reference arm runs and prints.
"""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    from dftpy_gb300 import systems
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, lr = bench.rank_info()
        t = bench.max_over_ranks(1.5 + rank, w, device="cpu")
        st = systems.config_al256(bench.rank_seed(r))
        pos = torch.tensor(st.positions.ravel())
        gathered = [torch.zeros_like(pos) for _ in range(w)]
        dist.all_gather(gathered, pos)
        buf = io.StringIO()

        class A:
            steps, warmup = 1, 0
        if r != 0:
            with redirect_stdout(buf):
                rc = bench.run_reference(A)
        else:
            rc = 0
        out.put((r, w, lr, t, float((gathered[0] - gathered[1]).abs().max()), rc, buf.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, lrank, t, dpos, rc, printed) in enumerate(res):
        assert (rank, world, lrank) == (r, 2, r)
        assert t == 2.5                      # max over ranks, on every rank
        assert dpos > 1e-3                   # the ranks' snapshots differ
        assert rc == 0
        if rank != 0:
            assert printed == ""             # non-zero ranks of the reference arm print nothing


def _shard_worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from dftpy_gb300 import batch
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sts = batch.alloy_batch(64)
        idx, mine = batch.shard(sts, rank, world)
        assert [s.name for s in mine] == ["alloy_%d" % i for i in idx]
        load = sum(batch.structure_cost(s) for s in mine)
        gathered = [None] * world
        dist.all_gather_object(gathered, (rank, idx, load))
        out.put(gathered)
    finally:
        dist.destroy_process_group()


def test_batch_shards_over_two_gloo_ranks():
    """The 64 alloy snapshots split over two ranks by longest-processing-time
    on the grid size: every structure is on exactly one rank, the union is
    the one-rank batch, every rank computed the same partition, and the
    larger load is within 4/3 of the ideal half."""
    import torch.multiprocessing as mp
    from dftpy_gb300 import batch
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    views = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert views[0] == views[1]
    (r0, idx0, load0), (r1, idx1, load1) = sorted(views[0])
    assert (r0, r1) == (0, 1)
    assert sorted(idx0 + idx1) == list(range(64)) and not set(idx0) & set(idx1)
    sts = batch.alloy_batch(64)
    one, _ = batch.shard(sts, 0, 1)
    assert one == list(range(64))
    total = sum(batch.structure_cost(s) for s in sts)
    assert load0 + load1 == total
    assert max(load0, load1) <= 4.0 / 3.0 * (total / 2.0)


def test_partition_lpt_properties():
    from dftpy_gb300 import batch
    rng = np.random.default_rng(3)
    for n, k in [(0, 3), (1, 4), (7, 7), (64, 8), (50, 3)]:
        costs = rng.integers(1, 100, n).tolist()
        parts, loads = batch.partition_lpt(costs, k)
        assert len(parts) == k
        assert sorted(i for p in parts for i in p) == list(range(n))
        for p, l in zip(parts, loads):
            assert l == sum(costs[i] for i in p)
        if n:
            assert max(loads) <= max(sum(costs) / k, max(costs)) * 4.0 / 3.0 + 1e-9
    with pytest.raises(ValueError):
        batch.partition_lpt([1, 2], 0)
