"""2-D partition of C = A B over ranks (one process per GPU).

Every block of C depends only on its row panel of A and its column panel of
B, so ranks need no reduction: each rank receives its panels as plain
copies into its own memory, computes its block with the GEMM it is given,
and the blocks are gathered.  The grid of ranks is the most square
factorisation of the world size.  The reference has no multi-device code;
on a pool with one GPU per box this runs as independent replicas.
"""
import math


def grid_shape(world):
    """(pr, pc) with pr * pc == world and pr <= pc as close as possible."""
    pr = int(math.isqrt(world))
    while world % pr:
        pr -= 1
    return pr, world // pr


def bounds(total, parts, idx):
    """[lo, hi) of part idx when `total` items are cut into `parts` parts
    that differ by at most one item."""
    q, r = divmod(total, parts)
    lo = idx * q + min(idx, r)
    return lo, lo + q + (1 if idx < r else 0)


def block_of(rank, world, m, n):
    """Rows and columns of C owned by `rank`."""
    pr, pc = grid_shape(world)
    i, j = divmod(rank, pc)
    return bounds(m, pr, i), bounds(n, pc, j)


def local_gemm(A, B, rank, world, gemm):
    """This rank's block of A @ B: gemm(A_panel, B_panel) -> block."""
    (r0, r1), (c0, c1) = block_of(rank, world, A.shape[0], B.shape[1])
    return gemm(A[r0:r1], B[:, c0:c1])


def assemble(blocks, world, m, n, empty):
    """Place the gathered blocks (indexed by rank) into `empty` (m, n, P)."""
    for rank, blk in enumerate(blocks):
        (r0, r1), (c0, c1) = block_of(rank, world, m, n)
        empty[r0:r1, c0:c1] = blk
    return empty
