"""Embedding output (the reference's EmbeddingWriter, IO/embedding_writer.h):
every row the device emits is an embedding, rows are distinct, their number
is the count and their set hash is the hash, both equal to the oracle's; the
task-range partitioning used when rows overflow one buffer yields the same
set; the text writer writes the same rows."""
import numpy as np
import pytest

import fsig_gb300 as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu

def fmix64_np(k):
    k = k.astype(np.uint64)
    with np.errstate(over="ignore"):
        k ^= k >> np.uint64(33)
        k *= np.uint64(0xFF51AFD7ED558CCD)
        k ^= k >> np.uint64(33)
        k *= np.uint64(0xC4CEB9FE1A85EC53)
        k ^= k >> np.uint64(33)
    return k


def set_hash(rows):
    """Order-independent hash of the rows, as include/fsig.h defines it."""
    if len(rows) == 0:
        return 0
    n = rows.shape[1]
    terms = fmix64_np((np.arange(n, dtype=np.uint64)[None, :] << np.uint64(32)) | rows.astype(np.uint64))
    with np.errstate(over="ignore"):
        inner = terms.sum(axis=1, dtype=np.uint64) + np.uint64(F.HASH_SEED)
        return int(fmix64_np(inner).sum(dtype=np.uint64))


def check_rows(g, q, rows):
    lab = np.asarray(g.labels)
    e = np.asarray(g.edges, np.int64).reshape(-1, 2)
    V = len(lab)
    edge_keys = set((e[:, 0] * V + e[:, 1]).tolist()) | set((e[:, 1] * V + e[:, 0]).tolist())
    assert rows.shape[1] == q.num_vertices
    assert np.all(lab[rows] == np.asarray(q.labels)[None, :])
    for a, b in np.asarray(q.edges).reshape(-1, 2).tolist():
        if a != b:
            keys = rows[:, a].astype(np.int64) * V + rows[:, b].astype(np.int64)
            assert all(k in edge_keys for k in keys.tolist())
    srt = np.sort(rows, axis=1)
    assert np.all(srt[:, 1:] != srt[:, :-1])  # injective
    assert len(np.unique(rows, axis=0)) == len(rows)  # distinct


@pytest.fixture(scope="module")
def small():
    """R-MAT, 10,000 vertices, 30,000 edges, 8 labels; a one-vertex query and
    random-walk queries of 2-5 vertices (930 to 155,578 embeddings)."""
    lab = F.gen_labels(10000, 8, "uniform", seed=7)
    g = F.gen_rmat(10000, 30000, 0.57, 0.19, 0.19, seed=7, labels=lab)
    off, adj = g.csr()
    qs = [F.Query(np.array([2], np.int32), np.zeros((0, 2), np.uint32))]
    qs += [F.gen_query(g, n, F.QUERY_INDUCED, seed=500 + i, csr=(off, adj)) for i, n in enumerate([2, 3, 4, 5])]
    want = [O.match(g.labels, off, adj, q.labels, q.edges)[:2] for q in qs]
    return g, qs, want


@pytest.mark.parametrize("algo", [F.ALGO_FSIG, F.ALGO_GSI])
def test_rows_are_the_embedding_set(engine, small, algo):
    g, qs, want = small
    engine.load_graph(g)
    for q, (c, h) in zip(qs, want):
        r, rows = engine.match_embeddings(q, algo)
        assert (r.count, r.hash) == (c, h)
        assert len(rows) == c
        check_rows(g, q, rows)
        assert set_hash(rows) == h


def test_overflowing_buffer_is_split_into_task_ranges(engine, small):
    g, qs, want = small
    engine.load_graph(g)
    q, (c, h) = max(zip(qs, want), key=lambda t: t[1][0])
    assert c > 2000
    _, full = engine.match_embeddings(q, F.ALGO_FSIG)
    r, rows = engine.match_embeddings(q, F.ALGO_FSIG, buffer_rows=max(c // 7, 1))
    assert (r.count, r.hash) == (c, h)
    assert len(rows) == c
    assert np.array_equal(np.unique(rows, axis=0), np.unique(full, axis=0))


def test_text_writer(engine, small, tmp_path):
    g, qs, want = small
    engine.load_graph(g)
    q, (c, h) = qs[3], want[3]
    path = tmp_path / "ans.txt"
    r = engine.write_embeddings(q, path, F.ALGO_FSIG)
    assert r.count == c
    text = path.read_text()
    rows = np.array([[int(x) for x in line.split()] for line in text.splitlines()], np.uint32).reshape(-1, q.num_vertices)
    assert len(rows) == c and set_hash(rows) == h


def test_no_embeddings_gives_no_rows(engine, small, tmp_path):
    g, _, _ = small
    engine.load_graph(g)
    # a label no data vertex has: no candidates, no embeddings
    q = F.Query(np.array([0, 9, 1], np.int32), np.array([[0, 1], [1, 2]], np.uint32))
    r, rows = engine.match_embeddings(q, F.ALGO_FSIG)
    assert r.count == 0 and rows.shape == (0, 3)
    path = tmp_path / "empty.txt"
    engine.write_embeddings(q, path, F.ALGO_FSIG)
    assert path.read_text() == ""
