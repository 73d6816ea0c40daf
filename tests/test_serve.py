"""Request server (gb300_server_*): host bookkeeping on the CPU, and on the
GPU the serving property -- every request's result is the same when it runs
alone and when it runs in a mix of concurrent, coalesced requests."""
import numpy as np
import pytest

from suitesparse_gb300 import matrices as M
from suitesparse_gb300 import serve as SV


def test_server_bookkeeping_without_work(lib):
    """Requests are queued, ordered per factor, coalesced, and every wait
    returns (on a machine without a GPU each request fails cleanly)."""
    S = SV.Server(nslots=2, budget_bytes=1 << 30, max_rhs=8)
    try:
        dims = (6, 5)
        mat = M.laplace2d(*dims, seed=3)
        S.factor(1, 10, 0, mat, M.grid_nd_perm(dims))
        B = M.rhs(mat[0], 2, 1)
        S.solve(2, 10, B)
        S.solve(3, 10, B[:, :1])
        S.solve(4, 99, B)                       # no such factor: fails, does not hang
        res = {r: S.wait(r) for r in (1, 2, 3, 4)}
        assert res[4][0] != 0
        for r in (1, 2, 3, 4):
            info = res[r][2]
            assert info["finish"] >= info["start"] >= info["arrival"] > 0
        st = S.stats()
        assert st["served"] == 4 and st["cached_patterns"] == 1
        with pytest.raises(RuntimeError):       # request ids are unique while pending
            S.solve(5, 10, B)
            S.solve(5, 10, B)
        S.wait(5)
    finally:
        S.close()


def _stream():
    return SV.make_stream(nreq=24, seed=7, rate=1e6, sides2d=(12, 40), sides3d=(6, 12),
                          ncached=3, p_reuse=0.5, p_solve=0.35, max_rhs=6)


def _backward_error(oracle_mod, rq, X):
    dims = rq["pat"]["dims"]
    gen = M.laplace2d if len(dims) == 2 else M.laplace3d
    # the matrix of the factor this solve ran against
    return oracle_mod, gen, dims


@pytest.mark.gpu
def test_same_result_alone_and_in_the_mix(lib, oracle_mod):
    stream = _stream()
    factors = {rq["fid"]: rq for rq in stream if rq["kind"] == "factor"}
    # alone: one request at a time
    S = SV.Server(nslots=4, budget_bytes=8 << 30, max_rhs=64)
    alone = {}
    try:
        seen = set()
        for rq in stream:
            if rq["kind"] == "factor":
                mat, perm = SV.request_inputs(rq)
                pid = rq["pat"]["pid"]
                S.factor(rq["req"], rq["fid"], pid, mat, None if pid in seen else perm)
                seen.add(pid)
            else:
                S.solve(rq["req"], rq["fid"], SV.request_inputs(rq))
            alone[rq["req"]] = S.wait(rq["req"])
    finally:
        S.close()
    # in the mix: everything submitted at once to 4 workers
    S = SV.Server(nslots=4, budget_bytes=8 << 30, max_rhs=64)
    try:
        mix, wall = SV.run_stream(S, stream, realtime=False)
        coalesced = S.stats()["coalesced"]
    finally:
        S.close()
    nsolve = nexact = 0
    for rq in stream:
        st_a, X_a, info_a = alone[rq["req"]]
        rec = mix[rq["req"]]
        assert st_a == 0 and rec["status"] == 0, (rq, st_a, rec["status"])
        if rq["kind"] != "solve":
            continue
        nsolve += 1
        # the factor this solve used: the latest factor request of that id
        # before it in the stream
        f = [q for q in stream if q["kind"] == "factor" and q["fid"] == rq["fid"]
             and q["req"] < rq["req"]][-1]
        mat, _ = SV.request_inputs(f)
        B = SV.request_inputs(rq)
        for X in (X_a, rec["X"]):
            be = oracle_mod.backward_error(*mat, X, B)
            assert be.max() <= 1e-12, (rq["req"], be.max())
        if rec["batch_cols"] == B.shape[1]:
            # not coalesced: the factorization (owner-computes, no atomics)
            # and the refined solve do the same arithmetic in the same order
            # alone and in the mix, so the solution is the same bit for bit
            assert np.array_equal(X_a, rec["X"]), rq["req"]
            nexact += 1
        else:
            # coalesced with other solves of the factor: the refinement ran
            # until every column converged, so this one may have taken an
            # extra step; both meet the target and agree to the forward
            # error it allows for these condition numbers
            rel = np.abs(X_a - rec["X"]).max() / np.abs(X_a).max()
            assert rel <= 1e-6, (rq["req"], rel)
    assert nsolve >= 4 and nexact >= 1


@pytest.mark.gpu
def test_evicted_factor_is_readmitted_for_its_solves(lib, oracle_mod):
    """A budget that holds about one factor: each new factor evicts the
    previous one (its A stays on the host); a solve against an evicted
    factor factorizes it again and gives the same solution, bit for bit,
    as the solve against the resident factor did; the charge of a resident
    factor is its measured device bytes."""
    mats = {}
    for fid, dims in enumerate(((40, 40), (36, 44), (12, 12, 12))):
        mats[fid] = (M.laplace2d(*dims, seed=fid) if len(dims) == 2
                     else M.laplace3d(dims[0], seed=fid)), M.grid_nd_perm(dims)
    S = SV.Server(nslots=1, budget_bytes=1 << 20, max_rhs=8)
    try:
        first = {}
        req = 0
        for fid, (mat, perm) in mats.items():
            S.factor(req, fid, fid, mat, perm)
            assert S.wait(req)[0] == 0
            st = S.stats()
            assert st["resident_factors"] == 1 and 0 < st["resident_bytes"]
            B = M.rhs(mat[0], 2, 10 + fid)
            S.solve(req + 1, fid, B)
            first[fid] = (B, S.wait(req + 1))
            assert first[fid][1][0] == 0
            req += 2
        st = S.stats()
        assert st["evictions"] >= 2 and st["evicted_kept"] == 2
        for fid, (mat, _) in mats.items():
            B, (_, X0, _) = first[fid]
            S.solve(req, fid, B)
            s1, X1, info = S.wait(req)
            req += 1
            assert s1 == 0, s1
            assert oracle_mod.backward_error(*mat, X1, B).max() <= 1e-12
            assert np.array_equal(X0, X1), fid
        assert S.stats()["readmissions"] >= 2
    finally:
        S.close()
