"""Serving: a stream of factor and solve requests through the library's
request server (gb300_server_* in include/cholmod_gb300.h).

The stream restates the serving workload: requests arrive as a Poisson
process; matrices are 2D 5-point and 3D 7-point grid Laplacians with
log-uniform coefficients; a share of the factor requests reuses one of a
few cached patterns with new values (each cached pattern owns one factor
id, refactorized in place: the server reuses the symbolic analysis, the plan
and the device factor), a share are solve-only requests against a resident
factor of a cached pattern with 1-32 right-hand sides (queued solves of one
factor are coalesced), the rest are factor requests of new patterns (a
factor id each, evicted least recently used under the byte budget).
Orderings are geometric nested dissection of the grids
(matrices.grid_nd_perm) given with a pattern's first request.  Matrix
values come from grid_matrix: new coefficients gathered into a pattern
cached per grid shape, so that a long stream's inputs are made as fast as
they arrive.
"""
import ctypes as C
import threading
import time

import numpy as np

from . import cholmod as CH
from . import matrices as M


def _lib():
    L = CH.lib()
    if not getattr(L, "_serve_sig", False):
        vp, i64, dp = C.c_void_p, C.c_int64, C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int64)
        sig = {
            "gb300_server_create": (vp, [C.c_int, i64, C.c_int]),
            "gb300_server_factor": (C.c_int, [vp, i64, i64, i64, i64, ip, ip, dp, ip, C.c_double]),
            "gb300_server_solve": (C.c_int, [vp, i64, i64, i64, C.c_int, dp, C.c_double]),
            "gb300_server_wait": (C.c_int, [vp, i64, dp, i64, dp]),
            "gb300_server_stats": (C.c_int, [vp, dp, C.c_int]),
            "gb300_server_destroy": (C.c_int, [vp]),
            "gb300_server_now": (C.c_double, []),
            "gb300_server_set_option": (C.c_int, [vp, C.c_int, i64]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        L._serve_sig = True
    return L


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Server:
    """Python handle of a gb300_server."""

    def __init__(self, nslots=4, budget_bytes=150 << 30, max_rhs=64):
        self.L = _lib()
        self.h = self.L.gb300_server_create(nslots, int(budget_bytes), max_rhs)
        if not self.h:
            raise RuntimeError("gb300_server_create failed")
        self.n = {}

    def now(self):
        return self.L.gb300_server_now()

    def factor(self, req, factor_id, pattern_id, mat, perm=None, arrival=None):
        n, Ap, Ai, Ax = mat
        Ap, Ai, Ax = _i64(Ap), _i64(Ai), _f64(Ax)
        pp = _i64(perm).ctypes.data_as(C.POINTER(C.c_int64)) if perm is not None else None
        st = self.L.gb300_server_factor(
            self.h, req, factor_id, pattern_id, n, Ap.ctypes.data_as(C.POINTER(C.c_int64)),
            Ai.ctypes.data_as(C.POINTER(C.c_int64)), Ax.ctypes.data_as(C.POINTER(C.c_double)),
            pp, self.now() if arrival is None else arrival)
        if st != 0:
            raise RuntimeError(f"factor request {req} rejected: status {st}")
        self.n[req] = (n, 0)

    def solve(self, req, factor_id, B, arrival=None):
        B = np.asfortranarray(_f64(B if B.ndim == 2 else B[:, None]))
        n, k = B.shape
        st = self.L.gb300_server_solve(self.h, req, factor_id, n, k,
                                       B.ctypes.data_as(C.POINTER(C.c_double)),
                                       self.now() if arrival is None else arrival)
        if st != 0:
            raise RuntimeError(f"solve request {req} rejected: status {st}")
        self.n[req] = (n, k)

    def wait(self, req):
        """(status, X or None, dict of times / backward error)"""
        n, k = self.n.pop(req)
        X = np.zeros((n, k), dtype=np.float64, order="F") if k else None
        out = (C.c_double * 7)()
        st = self.L.gb300_server_wait(
            self.h, req, X.ctypes.data_as(C.POINTER(C.c_double)) if k else None, n, out)
        info = dict(arrival=out[0], start=out[1], finish=out[2], berr=out[3],
                    iterations=int(out[4]), status=int(out[5]), batch_cols=int(out[6]))
        return st, X, info

    def stats(self):
        out = (C.c_double * 10)()
        self.L.gb300_server_stats(self.h, out, 10)
        keys = ("resident_bytes", "budget_bytes", "resident_factors", "cached_patterns",
                "evictions", "coalesced", "served", "readmissions", "evicted_kept",
                "evicted_host_bytes")
        return dict(zip(keys, list(out)))

    def set_option(self, option, value):
        """gb300_set_option on every worker's Common (e.g. GB300_OPT_PIVOT_LOG2
        = 0: every factorization takes the FP64 factor, the plain FP64 form)."""
        if not self.L.gb300_server_set_option(self.h, option, int(value)):
            raise RuntimeError(f"server option {option} refused")

    def close(self):
        if self.h:
            self.L.gb300_server_destroy(self.h)
            self.h = None


_grids = {}


def _grid_struct(dims):
    """Per grid shape: the lower CSC pattern of the Dirichlet grid Laplacian
    (column v: the diagonal, then the neighbours v + 1, v + nx, v + nx ny
    that exist, rows ascending) and the edge indices that form each stored
    value (diagonal: the 2 d incident edges, the ghost ones included;
    off-diagonal: minus the edge between the two nodes)."""
    key = tuple(int(d) for d in dims)
    if key in _grids:
        return _grids[key]
    nd = len(key)
    n = int(np.prod(key))
    coord = np.indices(key[::-1]).reshape(nd, -1)[::-1]     # coord[d][v], x fastest
    strides = np.cumprod((1,) + key[:-1])
    # flat edge index of direction d at node coordinate c (coordinate d in 0..dims[d])
    eoff, eshape = [], []
    tot = 0
    for d in range(nd):
        shp = list(key)
        shp[d] += 1
        eoff.append(tot)
        eshape.append(shp)
        tot += int(np.prod(shp))

    def edge(d, c):
        shp = eshape[d]
        flat = np.zeros(c.shape[1], dtype=np.int64)
        mul = 1
        for a in range(nd):
            flat += c[a] * mul
            mul *= shp[a]
        return eoff[d] + flat

    # entries per column: diagonal + one per existing forward neighbour
    has = [coord[d] < key[d] - 1 for d in range(nd)]
    cnt = 1 + sum(h.astype(np.int64) for h in has)
    Ap = np.zeros(n + 1, dtype=np.int64)
    Ap[1:] = np.cumsum(cnt)
    Ai = np.empty(int(Ap[-1]), dtype=np.int64)
    pos = Ap[:-1].copy()
    v = np.arange(n, dtype=np.int64)
    diag_pos = pos.copy()
    Ai[diag_pos] = v
    pos += 1
    lo_e, hi_e, off_pos, off_e = [], [], [], []
    for d in range(nd):
        lo_e.append(edge(d, coord))                       # edge before the node
        c2 = coord.copy()
        c2[d] += 1
        hi_e.append(edge(d, c2))                          # edge after the node
        m = has[d]
        off_pos.append(pos[m].copy())
        off_e.append(hi_e[d][m])
        Ai[pos[m]] = v[m] + strides[d]
        pos[m] += 1
    st = dict(n=n, Ap=Ap, Ai=Ai, E=tot, diag_pos=diag_pos, lo_e=lo_e, hi_e=hi_e,
              off_pos=off_pos, off_e=off_e)
    _grids[key] = st
    return st


def grid_matrix(dims, seed, lo=1e-2, hi=1e2, shift=0.0):
    """(n, Ap, Ai, Ax): the grid Laplacian of shape dims with edge
    conductivities log-uniform in [lo, hi] from seed (one uniform stream
    over every edge, ghost edges to the Dirichlet boundary included; numpy's
    PCG64 and exp, fast enough to make a stream's inputs as they arrive)."""
    st = _grid_struct(dims)
    u = np.random.default_rng(seed).random(st["E"])
    c = np.exp(np.log(lo) + u * (np.log(hi) - np.log(lo)))
    x = np.empty(len(st["Ai"]), dtype=np.float64)
    dg = np.full(st["n"], float(shift))
    for d in range(len(st["lo_e"])):
        dg += c[st["lo_e"][d]] + c[st["hi_e"][d]]
        x[st["off_pos"][d]] = -c[st["off_e"][d]]
    x[st["diag_pos"]] = dg
    return st["n"], st["Ap"], st["Ai"], x


def make_stream(nreq=200, seed=5, rate=200.0, sides2d=(32, 160), sides3d=(16, 40),
                ncached=16, p_reuse=0.6, p_solve=0.2, max_rhs=32):
    """A request stream: list of dicts with kind, arrival offset (s), ids and
    inputs' seeds.  Pattern ids 0..ncached-1 are the cached set, and cached
    pattern p is factor id p (refactorized in place by its reuse requests);
    solves go to a cached factor already requested; a new pattern gets a
    fresh pattern id and factor id."""
    rng = np.random.default_rng(seed)

    def new_pattern(pid):
        if rng.random() < 0.5:
            s = int(np.exp(rng.uniform(np.log(sides2d[0]), np.log(sides2d[1]))))
            return dict(pid=pid, dims=(s, s))
        s = int(np.exp(rng.uniform(np.log(sides3d[0]), np.log(sides3d[1]))))
        return dict(pid=pid, dims=(s, s, s))

    cached = [new_pattern(p) for p in range(ncached)]
    next_pid, next_fid = ncached, ncached
    resident = []                        # cached factor ids already requested
    t = 0.0
    out = []
    for r in range(nreq):
        t += rng.exponential(1.0 / rate)
        u = rng.random()
        if u < p_solve and resident:
            fid = resident[int(rng.integers(len(resident)))]
            out.append(dict(kind="solve", req=r, t=t, fid=fid, pat=cached[fid],
                            nrhs=int(rng.integers(1, max_rhs + 1)), seed=int(rng.integers(1 << 30))))
            continue
        if u < p_solve + p_reuse:
            pat = cached[int(rng.integers(ncached))]
            fid = pat["pid"]
            if fid not in resident:
                resident.append(fid)
        else:
            pat = new_pattern(next_pid)
            next_pid += 1
            fid = next_fid
            next_fid += 1
        out.append(dict(kind="factor", req=r, t=t, fid=fid, pat=pat,
                        seed=int(rng.integers(1 << 30))))
    return out


def request_inputs(rq, _cache={}):
    """Matrix (and ordering) of a factor request, or B of a solve request."""
    pat = rq["pat"]
    dims = pat["dims"]
    if rq["kind"] == "factor":
        mat = grid_matrix(dims, rq["seed"], lo=1e-2, hi=1e2)
        key = dims
        if key not in _cache:
            _cache[key] = M.grid_nd_perm(dims)
        return mat, _cache[key]
    n = int(np.prod(dims))
    return M.rhs(n, rq["nrhs"], rq["seed"] % 1000003)


def factor_weight(pat):
    """Estimated factor bytes of a request's pattern, for splitting streams
    across GPUs: nnz(L) of a nested-dissection factor grows as n log n on a
    2D grid and as n^(4/3) on a 3D grid."""
    n = float(np.prod(pat["dims"]))
    return n * np.log2(max(n, 2.0)) if len(pat["dims"]) == 2 else n ** (4.0 / 3.0)


def shard_stream(stream, world_size, rank):
    """This rank's requests of a stream split across world_size GPUs with no
    communication: factor ids are split by the estimated factor bytes of
    all their factor requests (a cached pattern's id is refactorized many
    times; batch.shard_systems, the same split on every rank) and every
    request follows its factor id, so a solve runs where its factor lives."""
    from .batch import shard_systems
    w = {}
    for q in stream:
        if q["kind"] == "factor":
            w[q["fid"]] = w.get(q["fid"], 0.0) + factor_weight(q["pat"])
    fids = sorted(w)
    part = shard_systems([w[f] for f in fids], world_size)[rank]
    mine = {fids[i] for i in part}
    return [q for q in stream if q["fid"] in mine]


def nd_orderings(stream, workers=0):
    """The nested-dissection ordering of every grid shape in the stream
    (computed once per shape; workers > 1: in a spawned process pool, so it
    may run after CUDA was initialized).  Fills request_inputs' cache."""
    shapes = sorted({tuple(q["pat"]["dims"]) for q in stream if q["kind"] == "factor"})
    cache = request_inputs.__defaults__[0]
    todo = [d for d in shapes if d not in cache]
    if workers > 1 and len(todo) > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(workers) as pool:
            for d, perm in zip(todo, pool.map(M.grid_nd_perm, todo)):
                cache[d] = perm
    else:
        for d in todo:
            cache[d] = M.grid_nd_perm(d)


def run_stream(server, stream, realtime=True, keep_x=None, producers=None):
    """Submit the stream (at its arrival times when realtime) from one
    thread, collect every request's result in another.  Producer threads
    (``producers``, default half the host's cores, 2 to 8) make the
    requests' inputs ahead of their arrival (at most 64 ahead; request i by
    producer i mod producers; numpy releases the interpreter lock in the
    array work, so they run side by side); a request whose inputs are late
    arrives when they are ready.
    keep_x: request ids whose solution is kept in the records (all when
    None).  Returns the per-request records and the wall time."""
    import os
    seen = set()
    nprod = producers or min(8, max(2, (os.cpu_count() or 2) // 2))
    made = {}                             # request index -> inputs
    cond = threading.Condition()
    next_i = [0]                          # the submitter's next request

    def producer(t):
        for i in range(t, len(stream), nprod):
            with cond:
                while i - next_i[0] >= 64:
                    cond.wait()
            inp = request_inputs(stream[i])
            with cond:
                made[i] = inp
                cond.notify_all()

    pts = [threading.Thread(target=producer, args=(t,), daemon=True) for t in range(nprod)]
    for pt in pts:
        pt.start()
    t0 = server.now()
    records = {}

    def submitter():
        for i, rq in enumerate(stream):
            with cond:
                while i not in made:
                    cond.wait()
                inp = made.pop(i)
                next_i[0] = i + 1
                cond.notify_all()
            if realtime:
                delay = t0 + rq["t"] - server.now()
                if delay > 0:
                    time.sleep(delay)
            arr = server.now()
            if rq["kind"] == "factor":
                mat, perm = inp
                pid = rq["pat"]["pid"]
                server.factor(rq["req"], rq["fid"], pid, mat, perm if pid not in seen else None,
                              arrival=arr)
                seen.add(pid)
            else:
                server.solve(rq["req"], rq["fid"], inp, arrival=arr)

    th = threading.Thread(target=submitter)
    th.start()
    for rq in stream:
        while rq["req"] not in server.n:
            time.sleep(1e-4)
        st, X, info = server.wait(rq["req"])
        info["status"] = st
        if keep_x is not None and rq["req"] not in keep_x:
            X = None if X is None else X.shape
        records[rq["req"]] = dict(kind=rq["kind"], X=X, **info)
    th.join()
    return records, server.now() - t0
