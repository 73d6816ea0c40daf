"""The batched workload: thousands of independent small SPD systems (2D
5-point Laplacians of a few distinct grid sides, each system with its own
coefficients) factorized and solved together.

A batch is the block-diagonal matrix diag(A_0, A_1, ...).  The symbolic
factor of each distinct pattern is analysed once (with the reference's AMD
permutation for that grid side, from the golden fixtures) and the batch's
symbolic factor is their concatenation (gb300_batch_analyze), so the numeric
factorization of the whole batch is one persistent launch over a forest and
the refinement checks every system's backward error separately.
"""
import os

import numpy as np

from . import cholmod as CH
from . import matrices as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def golden_perms(sides):
    """AMD permutations of the grid sides (reference analysis, fixtures)."""
    arrays = np.load(os.path.join(ROOT, "tests", "golden", "golden_arrays.npz"))
    return [arrays[f"c4_{s}_Perm"].astype(np.int64) for s in sides]


def c4_workload(nsys=4096, seed=3, systems=None):
    """sides (8 distinct), sys_pat (side index of each system), perms, and
    the systems' lower-triangular CSC matrices (only those of the indices in
    ``systems`` when given; ``pat`` still covers every system)."""
    sides, pat = M.batch_layout(nsys, seed)
    perms = golden_perms(sides)
    idx = range(nsys) if systems is None else systems
    mats = [M.batch_system(i, sides[pat[i]]) for i in idx]
    return sides, pat, perms, mats


def shard_systems(weights, world_size):
    """Split independent systems across ranks by weight (for a batch, the
    bytes of each system's factor), with no communication: every rank
    computes the same split from the same inputs.  Largest first, each to
    the least-loaded rank (ties: lower system index first, lower rank
    first).  Returns, per rank, its system indices in increasing order; the
    largest load exceeds the mean by at most one system's weight."""
    import heapq
    w = [float(x) for x in weights]
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    heap = [(0.0, r) for r in range(world_size)]
    out = [[] for _ in range(world_size)]
    for i in sorted(range(len(w)), key=lambda i: (-w[i], i)):
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + w[i], r))
    return [sorted(o) for o in out]


class Batch:
    """Symbolic factors of the patterns, the batch's symbolic factor and the
    block-diagonal matrix, owned by one cholmod_common."""

    def __init__(self, common, sides, pat, perms, mats):
        self.c = common
        self.Lpats = []
        for s, perm in zip(sides, perms):
            n, Ap, Ai, Ax = M.batch_system(0, s)
            A = CH.sparse(n, Ap, Ai, Ax, common)
            self.Lpats.append(CH.analyze_perm(A, perm, common))
            CH.free_sparse(A, common)
        self.L = CH.batch_analyze(self.Lpats, pat, common)
        self.n, Ap, Ai, Ax = M.block_diag_lower(mats)
        self.A = CH.sparse(self.n, Ap, Ai, Ax, common)
        self.offsets = np.cumsum([0] + [m[0] for m in mats]).astype(np.int64)

    def free(self):
        for L in self.Lpats + [self.L]:
            CH.free_factor(L, self.c)
        CH.free_sparse(self.A, self.c)
