"""Multi-process host path (world size 2, gloo on CPU): batch shards by graph,
max-over-ranks timing and the gather used by the bench's N > 1 runs."""

import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, per_rank, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    from gpu_bitruss_gb300 import gen, replicas
    from oracle import oracle as O
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, _ = replicas.dist_env()
        assert (r, w) == (rank, world)
        mine = replicas.batch_shard(per_rank, r)
        summary = {}
        for i in mine:
            u, v = gen.er(20 + i, 25 + i, 150 + 10 * i, seed=300 + i)
            res, lv, _ = O.msp(O.build_csr(u, v), 1, O.MSP_REF)
            summary[i] = (int(res.sum()), lv)
        replicas.barrier()
        t = replicas.max_over_ranks(1.5 + rank)  # the slower rank decides
        allsum = replicas.gather(summary)
        if rank == 0:
            q.put((t, allsum))
    finally:
        dist.destroy_process_group()


def test_batch_shards_and_rank_reductions_on_gloo(oracle_mod):
    import torch.multiprocessing as mp
    from gpu_bitruss_gb300 import gen
    world, per_rank = 2, 3
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, per_rank, q)) for r in range(world)]
    for p in procs:
        p.start()
    t, allsum = q.get(timeout=180)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert t == 2.5
    seen = [i for d in allsum for i in d]
    assert sorted(seen) == list(range(world * per_rank))  # disjoint, complete
    O = oracle_mod
    for d in allsum:
        for i, (s, lv) in d.items():
            u, v = gen.er(20 + i, 25 + i, 150 + 10 * i, seed=300 + i)
            res, want_lv, _ = O.msp(O.build_csr(u, v), 1, O.MSP_REF)
            assert (s, lv) == (int(res.sum()), want_lv)


def test_single_process_fallbacks():
    sys.path.insert(0, ROOT)
    from gpu_bitruss_gb300 import replicas
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.gather({"a": 1}) == [{"a": 1}]
    assert replicas.batch_shard(4, 2) == [8, 9, 10, 11]
    assert replicas.batch_shard(4, 2, total=10) == [8, 9]
