"""The graph store without a segment table (FSIG_SEGMENTS_ROWS).

A store built with the dense table keeps, for every row, the start of every
label's segment (V x (L+1) words) and the caller id of every adjacency entry;
one built without it finds a segment by binary search in the row and a
leaf's caller id by one lookup.  Every result must be the same either way:
counts, hashes and per-depth counts of all three algorithms through the
single-query, batched (with and without a CUDA graph, with refinement) and
task-range paths, filter flags, emitted embeddings, and a graph cache saved
from a store without the table.  Counts and hashes are also checked against
the oracle.  The automatic choice takes the table for few labels and goes
without it when the table would outweigh the adjacency.
"""
import numpy as np
import pytest

import fsig_gb300 as F
from fsig_gb300.workloads import pattern
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ALGOS = (F.ALGO_FSIG, F.ALGO_GSI, F.ALGO_FUSED)


def _graph(kind):
    if kind == "rmat3":  # R-MAT 2^12 / 2^15, 3 uniform labels: heavy enumeration
        lab = F.gen_labels(1 << 12, 3, "uniform", seed=9)
        return F.gen_rmat(1 << 12, 1 << 15, 0.57, 0.19, 0.19, seed=9, labels=lab)
    if kind == "rmat1024":  # R-MAT 2^13 / 2^16, 1,024 Zipf labels: the table would be 8.4 M words
        lab = F.gen_labels(1 << 13, 1024, "zipf", seed=4)
        return F.gen_rmat(1 << 13, 1 << 16, 0.57, 0.19, 0.19, seed=4, labels=lab)
    return F.gen_rmat(1 << 9, 1 << 12, 0.57, 0.19, 0.19, seed=3)  # unlabeled


@pytest.fixture(scope="module", params=["rmat3", "rmat1024", "unlabeled"])
def case(request):
    g = _graph(request.param)
    off, adj = g.csr()
    if request.param == "unlabeled":
        qs = [pattern("house"), pattern("c5"), pattern("k4_pendant")]
    else:
        # at most a few 10^8 embeddings each (the oracle's share of the time)
        qs = [F.gen_query(g, n, F.QUERY_DENSE, seed=70 + n, csr=(off, adj)) for n in (3, 4, 5, 6)]
        qs += [F.gen_query(g, n, F.QUERY_SPARSE, seed=70 + n, csr=(off, adj)) for n in (3, 4, 5)]
    want = [O.match(g.labels, off, adj, q.labels, q.edges)[:2] for q in qs]
    return request.param, g, qs, want


def _results(e, qs):
    out = []
    for q in qs:
        for algo in ALGOS:
            r = e.match(q, algo)
            out.append((algo, r.status, r.count, r.hash, tuple(r.level_counts)))
    for use_graph in (True, False):
        for refine in (0, 2):
            rs = e.match_batch(qs, algo=F.ALGO_FUSED, use_graph=use_graph, refine_iters=refine)
            out += [("batch", use_graph, refine, r.status, r.count, r.hash) for r in rs]
    return out


def _engine(mode):
    e = F.Engine(0, arena_bytes=2 << 30)
    e.set_segment_index(mode)
    return e


def test_rows_index_gives_the_table_results(case):
    name, g, qs, want = case
    with _engine(F.SEGMENTS_TABLE) as et, _engine(F.SEGMENTS_ROWS) as er:
        et.load_graph(g)
        er.load_graph(g)
        assert et.graph_layout()["segment_index"] == F.SEGMENTS_TABLE
        assert er.graph_layout()["segment_index"] == F.SEGMENTS_ROWS
        assert er.graph_layout()["bytes"] < et.graph_layout()["bytes"]
        got_t, got_r = _results(et, qs), _results(er, qs)
        assert got_r == got_t
        for q, (c, h) in zip(qs, want):
            r = er.match(q, F.ALGO_GSI)
            assert (r.status, r.count, r.hash) == (0, c, h)
        for q in qs:
            for algo in ALGOS:
                for refine in (0, 2):
                    assert np.array_equal(er.filter(q, algo, refine), et.filter(q, algo, refine))


def test_rows_index_ranges_and_embeddings(case):
    name, g, qs, want = case
    with _engine(F.SEGMENTS_ROWS) as e:
        e.load_graph(g)
        for q, (c, h) in zip(qs, want):
            _, T = e.match_range(q, F.ALGO_FUSED, 0, 0, split_len=32)
            cuts = sorted({0, T, T // 3, T // 2})
            count = hsum = 0
            for a, b in zip(cuts[:-1], cuts[1:]):
                r, _ = e.match_range(q, F.ALGO_FUSED, a, b, split_len=32)
                count += r.count
                hsum = (hsum + r.hash) % (1 << 64)
            assert (count, hsum) == (c, h)
            if c <= 200_000:
                r, rows = e.match_embeddings(q, F.ALGO_GSI)
                assert (r.count, r.hash, len(rows)) == (c, h, c)
                lab = np.asarray(g.labels)
                if c:
                    assert np.all(lab[rows] == np.asarray(q.labels)[None, :])
                    assert len(np.unique(rows, axis=0)) == c


def test_rows_index_graph_cache(case, tmp_path):
    name, g, qs, want = case
    path = tmp_path / "rows.fsigcache"
    with _engine(F.SEGMENTS_ROWS) as e:
        e.load_graph(g)
        e.save_graph_cache(path)
    with _engine(F.SEGMENTS_TABLE) as e:  # a cache keeps the index it was saved with
        e.load_graph_cache(path)
        assert e.graph_layout()["segment_index"] == F.SEGMENTS_ROWS
        for q, (c, h) in zip(qs, want):
            r = e.match(q, F.ALGO_FSIG)
            assert (r.status, r.count, r.hash) == (0, c, h)


def test_automatic_choice():
    with _engine(F.SEGMENTS_AUTO) as e:
        e.load_graph(_graph("rmat3"))
        assert e.graph_layout()["segment_index"] == F.SEGMENTS_TABLE
        e.load_graph(_graph("rmat1024"))
        assert e.graph_layout()["segment_index"] == F.SEGMENTS_ROWS
        with pytest.raises(F.FsigError) as ei:
            e.set_segment_index(3)
        assert ei.value.status == F.EINVAL
