"""Unlabeled counting (the config-3 case, graph_type = 0) at reduced scale:
R-MAT graphs (seed 3) with 2^10 vertices and 2^13 edges (up to 7e8
embeddings per pattern) and with 2^8 vertices and 2^11 edges (the oracle
checks every pattern there), no labels, and the five 5-vertex patterns -- K4 plus a pendant vertex, the 5-cycle, the house and
two seeded random connected graphs.  Skewed degree lists stress the segment
searches.  Pins: the K4+pendant identity (its count is the sum over ordered
K4 embeddings of deg(image of the attach vertex) - 3, with the K4 embeddings
taken from the embedding output; and at 2^12 vertices and 2^16 edges, the
config-3 density, from the oracle's clique listing), agreement of the three
algorithms and of the batched path, and the oracle where it finishes
quickly."""
import numpy as np
import pytest

import fsig_gb300 as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def pattern(edges):
    return F.Query(np.zeros(5, np.int32), np.asarray(edges, np.uint32))


def random_connected(seed):
    rng = np.random.default_rng(seed)
    while True:
        e = {(i, j) for i in range(5) for j in range(i + 1, 5) if rng.random() < 0.5}
        adj = {i: set() for i in range(5)}
        for a, b in e:
            adj[a].add(b)
            adj[b].add(a)
        seen, todo = {0}, [0]
        while todo:
            for w in adj[todo.pop()]:
                if w not in seen:
                    seen.add(w)
                    todo.append(w)
        if len(seen) == 5:
            return sorted(e)


PATTERNS = {
    "k4_pendant": [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3), (0, 4)],
    "c5": [(0, 1), (1, 2), (2, 3), (3, 4), (4, 0)],
    "house": [(0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (1, 4)],
    "random_a": random_connected(31),
    "random_b": random_connected(32),
}


@pytest.fixture(scope="module")
def rmat():
    g = F.gen_rmat(1 << 10, 1 << 13, 0.57, 0.19, 0.19, seed=3)
    off, adj = g.csr()
    return g, off, adj


@pytest.fixture(scope="module")
def tiny():
    g = F.gen_rmat(1 << 8, 1 << 11, 0.57, 0.19, 0.19, seed=3)
    off, adj = g.csr()
    return g, off, adj


def test_k4_pendant_identity(engine, rmat):
    g, off, adj = rmat
    engine.load_graph(g)
    k4 = F.Query(np.zeros(4, np.int32), np.asarray(PATTERNS["k4_pendant"][:6], np.uint32))
    r4, rows = engine.match_embeddings(k4, F.ALGO_FSIG)
    assert len(rows) == r4.count > 0
    deg = np.diff(off.astype(np.int64))
    expect = int((deg[rows[:, 0]] - 3).sum())
    r = engine.match(pattern(PATTERNS["k4_pendant"]), F.ALGO_FSIG)
    assert r.count == expect


def test_k4_pendant_identity_at_config3_density(engine):
    """R-MAT 2^12 / 2^16 (16 edges per vertex, as in config 3): the engine's
    K4 count (2.4e8 embeddings) and K4+pendant count (1.0e11) against the
    oracle's clique listing and the identity 6 * sum over K4s of the sum of
    (deg - 3) -- a pin at a scale the backtracking oracle does not reach."""
    g = F.gen_rmat(1 << 12, 1 << 16, 0.57, 0.19, 0.19, seed=3)
    off, adj = g.csr()
    k4, pend = O.k4_pendant(off, adj)
    engine.load_graph(g)
    q4 = F.Query(np.zeros(4, np.int32), np.asarray(PATTERNS["k4_pendant"][:6], np.uint32))
    r4 = engine.match(q4, F.ALGO_GSI)
    assert (r4.status, r4.count) == (0, 24 * k4)
    r = engine.match(pattern(PATTERNS["k4_pendant"]), F.ALGO_GSI)
    assert (r.status, r.count) == (0, pend)


@pytest.mark.parametrize("name", sorted(PATTERNS))
def test_algorithms_and_batch_agree(engine, rmat, name):
    g, off, adj = rmat
    engine.load_graph(g)
    q = pattern(PATTERNS[name])
    res = [engine.match(q, a) for a in (F.ALGO_FSIG, F.ALGO_GSI, F.ALGO_FUSED)]
    res += engine.match_batch([q] * 3, algo=F.ALGO_FUSED, use_graph=True)
    assert len({(r.count, r.hash) for r in res}) == 1
    assert res[0].count > 0


@pytest.mark.parametrize("name", sorted(PATTERNS))
def test_patterns_match_oracle(engine, tiny, name):
    g, off, adj = tiny
    engine.load_graph(g)
    q = pattern(PATTERNS[name])
    c, h, _ = O.match(g.labels, off, adj, q.labels, q.edges)
    for a in (F.ALGO_FSIG, F.ALGO_GSI, F.ALGO_FUSED):
        r = engine.match(q, a)
        assert (r.count, r.hash) == (c, h)
