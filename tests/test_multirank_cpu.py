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
