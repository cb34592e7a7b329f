"""The N > 1 path on CPU: world-size-2 gloo process groups.  Matching shards
by query across replicas with no data-path collective; the only exchange is
the host-side sum of counts and set hashes (mod 2^64) and the max of the
ranks' times, which bench.py's Dist does.  Each rank here matches its shard
with the oracle (the GPU engine has no CPU path)."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    try:
        _work(rank, world, port, out)
    except BaseException as exc:  # report instead of leaving the parent waiting
        out.put((rank, "error", repr(exc), 0.0, []))
        raise


def _work(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    from fsig_gb300 import workloads as W
    import fsig_gb300 as F
    from oracle import oracle as O
    d = bench.Dist()
    lab = F.gen_labels(2000, 4, "uniform", seed=3)
    g = F.gen_rmat(2000, 8000, 0.57, 0.19, 0.19, seed=3, labels=lab)
    off, adj = g.csr()
    qs = [F.gen_query(g, 4, F.QUERY_INDUCED, seed=70 + i, csr=(off, adj)) for i in range(12)]
    mine = qs[rank::world]  # shard by query
    c = h = 0
    for q in mine:
        cnt, hs = O.match(g.labels, off, adj, q.labels, q.edges)[:2]
        c += cnt
        h = (h + hs) % (1 << 64)
    # counts fit a double exactly here; hashes are exchanged as two 32-bit halves
    tot_c = d.sum(c)
    lo = d.sum(h & 0xFFFFFFFF)
    hi = d.sum(h >> 32)
    tot_h = (int(lo) + (int(hi) << 32)) % (1 << 64)
    mx = d.max(float(rank + 1))
    d.barrier()
    out.put((rank, int(tot_c), tot_h, mx, W.rank_order(4, rank)))
    d.close()


@pytest.fixture(scope="module")
def two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(res)


def test_shard_sums_equal_single_process(two_ranks):
    sys.path.insert(0, str(ROOT))
    import fsig_gb300 as F
    from oracle import oracle as O
    lab = F.gen_labels(2000, 4, "uniform", seed=3)
    g = F.gen_rmat(2000, 8000, 0.57, 0.19, 0.19, seed=3, labels=lab)
    off, adj = g.csr()
    c = h = 0
    for i in range(12):
        q = F.gen_query(g, 4, F.QUERY_INDUCED, seed=70 + i, csr=(off, adj))
        cnt, hs = O.match(g.labels, off, adj, q.labels, q.edges)[:2]
        c += cnt
        h = (h + hs) % (1 << 64)
    for rank, tc, th, _, _ in two_ranks:
        assert tc != "error", th
        assert (tc, th) == (c, h)


def test_max_over_ranks(two_ranks):
    assert [r[3] for r in two_ranks] == [2.0, 2.0]


def test_ranks_start_at_distinct_batches(two_ranks):
    """Replicas run the manifest's batches, rank r starting at batch r, so
    that at any step the ranks work on different queries."""
    s0, s1 = two_ranks[0][4], two_ranks[1][4]
    assert s0 == [0, 1, 2, 3] and s1 == [1, 2, 3, 0]
