"""Seeded synthetic workloads: determinism, distinct simple edges, queries
that embed at their source vertices."""
import numpy as np
import pytest

import fsig_gb300 as F
from oracle import oracle as O


def test_rmat_distinct_and_deterministic():
    g1 = F.gen_rmat(10000, 50000, seed=1)
    g2 = F.gen_rmat(10000, 50000, seed=1, threads=3)
    assert np.array_equal(g1.edges, g2.edges)  # independent of the thread count
    e = g1.edges
    assert e.shape == (50000, 2)
    assert (e[:, 0] < e[:, 1]).all()
    keys = e[:, 0].astype(np.uint64) << np.uint64(32) | e[:, 1]
    assert len(np.unique(keys)) == len(keys)
    assert e.max() < 10000


def test_chung_lu_power_law():
    g = F.gen_chung_lu(50000, 200000, 2.1, seed=2)
    deg = np.bincount(g.edges.reshape(-1), minlength=50000)
    assert deg.sum() == 400000
    assert deg.max() > 20 * deg.mean()
    assert deg.max() <= 2.0 * np.sqrt(400000) + 50


def test_zipf_labels():
    lab = F.gen_labels(100000, 16, "zipf", seed=2)
    c = np.bincount(lab, minlength=16)
    assert c[0] > c[1] > c[3] > c[15] > 0
    assert abs(c[0] / c[1] - 2.0) < 0.2


@pytest.mark.parametrize("mode", [F.QUERY_INDUCED, F.QUERY_DENSE, F.QUERY_SPARSE])
def test_queries_embed_at_source(mode):
    lab = F.gen_labels(20000, 8, "zipf", seed=3)
    g = F.gen_chung_lu(20000, 80000, 2.1, seed=3, labels=lab)
    off, adj = g.csr()
    for s in range(5):
        n = 8
        q = F.gen_query(g, n, mode, seed=s, csr=(off, adj))
        m = len(q.edges)
        if mode == F.QUERY_DENSE:
            assert 8 * m > min(12 * n, 3 * n * (n - 1))
        if mode == F.QUERY_SPARSE:
            assert 2 * m <= 3 * n
        assert (g.labels[q.source] == q.labels).all()
        for a, b in q.edges.tolist():
            x, y = q.source[a], q.source[b]
            assert y in adj[off[x]:off[x + 1]]
        assert len(set(q.source.tolist())) == n


def test_tve_roundtrip(tmp_path):
    lab = F.gen_labels(500, 5, "uniform", seed=4)
    g = F.gen_rmat(500, 2000, seed=4, labels=lab)
    p = tmp_path / "g.graph"
    g.write_tve(p)
    assert not p.read_text().endswith("\n")
    d = O.read_tve(p)
    g2 = F.read_graph(p)
    assert d["E"] == 2000 and np.array_equal(d["labels"], lab)
    assert np.array_equal(g2.edges, g.edges)
    (tmp_path / "h.graph").write_text(p.read_text() + "\n")
    g3 = F.read_graph(tmp_path / "h.graph")
    assert len(g3.edges) == 2001 and (g3.edges[-1] == g3.edges[-2]).all()
