"""Batches shard across GPUs by independent systems, with no collective on
the data path: every rank computes the same split of the systems by factor
bytes (batch.shard_systems) and factors its share as its own batch; only the
timing uses the process group (barrier, max over ranks).  On the CPU: the
split's properties, and two gloo ranks that compute it independently and
agree, with bench.py's barrier and max-over-ranks reduction."""
import json
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from suitesparse_gb300 import batch as BT  # noqa: E402
from suitesparse_gb300 import matrices as M  # noqa: E402


def c4_weights(nsys):
    gold = json.load(open(os.path.join(ROOT, "tests", "golden", "golden.json")))
    sides, pat = M.batch_layout(nsys, 3)
    return [gold[f"c4_{sides[q]}"]["xsize"] for q in pat]


@pytest.mark.parametrize("ws", [1, 2, 3, 8])
def test_split_covers_balances_and_repeats(ws):
    w = c4_weights(4096 * ws)
    parts = BT.shard_systems(w, ws)
    assert len(parts) == ws
    allidx = np.concatenate([np.asarray(p, np.int64) for p in parts])
    assert len(allidx) == len(w) and len(np.unique(allidx)) == len(w)
    for p in parts:
        assert list(p) == sorted(p)
    loads = np.array([sum(w[i] for i in p) for p in parts], np.float64)
    assert loads.max() - loads.mean() <= max(w)
    assert loads.max() <= 1.01 * loads.mean()
    assert BT.shard_systems(w, ws) == parts          # the same on every call


def test_split_edge_cases():
    assert BT.shard_systems([], 2) == [[], []]
    assert BT.shard_systems([5.0], 3) == [[0], [], []]
    # equal weights: round robin by rank, lower index first
    assert BT.shard_systems([1, 1, 1, 1], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        BT.shard_systems([1.0], 0)


def _rank_main(rank, ws, port, nsys):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    os.environ["RANK"] = str(rank)
    os.environ["WORLD_SIZE"] = str(ws)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        import bench
        mine = BT.shard_systems(c4_weights(nsys), ws)[rank]
        every = [None] * ws
        dist.all_gather_object(every, mine)
        # the split each rank computed alone agrees with every other rank's
        assert every[rank] == mine
        full = BT.shard_systems(c4_weights(nsys), ws)
        assert every == full
        bench.barrier(dist)
        assert bench.max_over_ranks(dist, 10.0 + rank) == 10.0 + (ws - 1)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_without_exchange():
    mp = pytest.importorskip("torch.multiprocessing")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.spawn(_rank_main, args=(2, port, 4096 * 2), nprocs=2, join=True)


@pytest.mark.parametrize("ws", [2, 3])
def test_request_stream_split(ws):
    """Request streams split by factor id: the ranks' shares partition the
    stream, every solve lands on the rank of its factor, and the estimated
    factor bytes are balanced."""
    from suitesparse_gb300 import serve as SV
    stream = SV.make_stream(nreq=300 * ws, seed=5, rate=100.0 * ws, sides2d=(32, 256),
                            sides3d=(16, 48), ncached=16, p_reuse=0.6, p_solve=0.2,
                            max_rhs=32)
    shares = [SV.shard_stream(stream, ws, r) for r in range(ws)]
    reqs = sorted(q["req"] for sh in shares for q in sh)
    assert reqs == sorted(q["req"] for q in stream)
    home = {}
    for r, sh in enumerate(shares):
        for q in sh:
            if q["kind"] == "factor":
                home[q["fid"]] = r
    for r, sh in enumerate(shares):
        for q in sh:
            assert home[q["fid"]] == r
    w = [sum(SV.factor_weight(q["pat"]) for q in sh if q["kind"] == "factor") for sh in shares]
    # the unit of the split is a factor id with all its factor requests (a
    # cached pattern's id is refactorized many times)
    per_fid = {}
    for q in stream:
        if q["kind"] == "factor":
            per_fid[q["fid"]] = per_fid.get(q["fid"], 0.0) + SV.factor_weight(q["pat"])
    assert max(w) - np.mean(w) <= max(per_fid.values())
    assert SV.shard_stream(stream, ws, 1) == shares[1]
