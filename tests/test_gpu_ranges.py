"""fsig_match_range: a query matched in pieces of its root-task space.

Ranges that partition the task space add up to the whole query's count and
set hash (hashes modulo 2^64) and per-depth counts, for every algorithm and
cut; the space's size does not depend on the range asked for; an empty range
finds nothing; a range running past the end is clipped; a reversed range is
refused.  The whole-query results are checked against the oracle.  (The
reference cuts one query's work into blocks too, to bound memory:
MMatch::extend_embeddings_recursively, match/MMatch.cu:1834-1985.)
"""
import numpy as np
import pytest

import fsig_gb300 as F
from fsig_gb300.workloads import pattern
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graph():
    lab = F.gen_labels(1 << 12, 3, "uniform", seed=9)
    g = F.gen_rmat(1 << 12, 1 << 15, 0.57, 0.19, 0.19, seed=9, labels=lab)
    off, adj = g.csr()
    qs = [F.gen_query(g, n, F.QUERY_DENSE, seed=90 + n, csr=(off, adj)) for n in (4, 5, 6)]
    return g, off, adj, qs


def test_ranges_partition_the_query(engine, graph):
    g, off, adj, qs = graph
    engine.load_graph(g)
    rng = np.random.default_rng(5)
    for q in qs:
        c0, h0, _ = O.match(g.labels, off, adj, q.labels, q.edges)
        for algo in (F.ALGO_FSIG, F.ALGO_GSI, F.ALGO_FUSED):
            full, T = engine.match_range(q, algo, 0, 0xFFFFFFFF)
            assert (full.status, full.count, full.hash) == (0, c0, h0)
            empty, T0 = engine.match_range(q, algo, 0, 0)
            assert T0 == T > 0 and empty.count == 0 and empty.hash == 0
            for split_len in (0, 32):
                _, Ts = engine.match_range(q, algo, 0, 0, split_len=split_len)
                cuts = sorted({0, Ts, *rng.integers(0, Ts, 6).tolist()})
                count = hsum = 0
                levels = np.zeros(q.num_vertices, np.uint64)
                for a, b in zip(cuts[:-1], cuts[1:]):
                    r, Tr = engine.match_range(q, algo, a, b, split_len=split_len)
                    assert Tr == Ts and r.status == 0
                    count += r.count
                    hsum = (hsum + r.hash) % (1 << 64)
                    levels += np.asarray(r.level_counts, np.uint64)
                assert (count, hsum) == (c0, h0)
                assert levels.tolist() == full.level_counts
            tail, _ = engine.match_range(q, algo, T - 1, T + 1000)
            last, _ = engine.match_range(q, algo, T - 1, T)
            assert (tail.count, tail.hash) == (last.count, last.hash)


def test_unlabeled_pattern_in_pieces(engine):
    g = F.gen_rmat(1 << 9, 1 << 12, 0.57, 0.19, 0.19, seed=3)
    off, adj = g.csr()
    engine.load_graph(g)
    q = pattern("house")
    c0, h0, _ = O.match(g.labels, off, adj, q.labels, q.edges)
    _, T = engine.match_range(q, F.ALGO_GSI, 0, 0)
    count = hsum = 0
    for a in range(0, T, 97):
        r, _ = engine.match_range(q, F.ALGO_GSI, a, a + 97)
        count += r.count
        hsum = (hsum + r.hash) % (1 << 64)
    assert (count, hsum) == (c0, h0)


def test_reversed_range_is_refused(engine, graph):
    g, off, adj, qs = graph
    engine.load_graph(g)
    with pytest.raises(F.FsigError) as ei:
        engine.match_range(qs[0], F.ALGO_GSI, 5, 4)
    assert ei.value.status == F.EINVAL
