"""The 2-D C partition over two CPU ranks (gloo): each rank computes its
block with the oracle's plain GEMM, the blocks are gathered, and the
result equals the single-process product bit for bit."""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import pkg


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import oracle
    from conftest import pkg as _pkg
    shard, inputs = _pkg("shard"), _pkg("inputs")
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    P, A, B = inputs.workload("qd1024", 13, 11, 9)
    blk = shard.local_gemm(A, B, rank, world,
                           lambda a, b: oracle.gemm_plain(P, a, b, a.shape[0], b.shape[1], a.shape[1]))
    gathered = [None] * world
    dist.all_gather_object(gathered, blk)
    if rank == 0:
        C = shard.assemble(gathered, world, 13, 11, np.zeros((13, 11, P)))
        out.put(C)
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_gemm_matches_single(world, orc):
    import socket
    with socket.socket() as s_:
        s_.bind(("127.0.0.1", 0))
        port = s_.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p_ in procs:
        p_.start()
    C = q.get(timeout=120)
    for p_ in procs:
        p_.join(timeout=60)
        assert p_.exitcode == 0
    inputs = pkg("inputs")
    P, A, B = inputs.workload("qd1024", 13, 11, 9)
    assert np.array_equal(C, orc.gemm_plain(P, A, B, 13, 11, 9))


def test_partition_covers_c_exactly():
    shard = pkg("shard")
    for world in (1, 2, 3, 4, 6, 8):
        cover = np.zeros((37, 29), dtype=int)
        for r in range(world):
            (r0, r1), (c0, c1) = shard.block_of(r, world, 37, 29)
            cover[r0:r1, c0:c1] += 1
        assert np.all(cover == 1)
