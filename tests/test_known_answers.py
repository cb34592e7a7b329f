"""Closed-form and brute-force pins of the oracle's matching semantics:
injective, label-preserving, non-induced embeddings with automorphic images
counted separately (match/GSI_kernels.cuh:199-213, MMatch_kernels.cuh:641-654),
and the order-independent set hash."""
import itertools
import math

import numpy as np
import pytest

import fsig_gb300 as F
from oracle import oracle as O

M64 = (1 << 64) - 1


def fmix64(k):
    k &= M64
    k ^= k >> 33
    k = (k * 0xFF51AFD7ED558CCD) & M64
    k ^= k >> 33
    k = (k * 0xC4CEB9FE1A85EC53) & M64
    k ^= k >> 33
    return k


def csr_of(V, edges):
    return F.Graph(np.zeros(V, np.int32), np.asarray(edges, np.uint32).reshape(-1, 2)).csr()


def count(V, edges, qn, qedges, labels=None, qlabels=None):
    off, adj = csr_of(V, edges)
    lab = np.zeros(V, np.int32) if labels is None else np.asarray(labels, np.int32)
    ql = np.zeros(qn, np.int32) if qlabels is None else np.asarray(qlabels, np.int32)
    c, h, lv = O.match(lab, off, adj, ql, np.asarray(qedges, np.uint32))
    return c


def complete(n):
    return [(i, j) for i in range(n) for j in range(i + 1, n)]


def path(k):
    return [(i, i + 1) for i in range(k - 1)]


def cycle(k):
    return path(k) + [(k - 1, 0)]


@pytest.mark.parametrize("n", [4, 5, 7])
def test_complete_graph(n):
    assert count(n, complete(n), 3, cycle(3)) == n * (n - 1) * (n - 2)
    assert count(n, complete(n), 4, complete(4)) == math.perm(n, 4)
    for k in range(2, n + 1):
        assert count(n, complete(n), k, path(k)) == math.perm(n, k)


@pytest.mark.parametrize("N", [5, 8, 11])
def test_cycle_graph(N):
    for k in range(2, N):
        assert count(N, cycle(N), k, path(k)) == 2 * N
    assert count(N, cycle(N), N, cycle(N)) == 2 * N
    assert count(N, cycle(N), 3, cycle(3)) == 0


def test_star():
    d = 6
    star = [(0, i) for i in range(1, d + 1)]
    for k in range(2, d + 1):
        q = [(0, i) for i in range(1, k + 1)]
        assert count(d + 1, star, k + 1, q) == math.perm(d, k)
    assert count(d + 1, star, 2, [(0, 1)]) == 2 * d


def test_labeled_bipartite():
    a, b = 4, 3
    edges = [(i, a + j) for i in range(a) for j in range(b)]
    lab = [0] * a + [1] * b
    assert count(a + b, edges, 2, [(0, 1)], lab, [0, 1]) == a * b
    assert count(a + b, edges, 3, [(0, 1), (1, 2)], lab, [0, 1, 0]) == b * a * (a - 1)
    assert count(a + b, edges, 2, [(0, 1)], lab, [0, 0]) == 0
    assert count(a + b, edges, 1, [], lab, [1]) == b


def brute(V, edges, lab, qn, qedges, qlab):
    es = set()
    for x, y in edges:
        if x != y:
            es.add((x, y))
            es.add((y, x))
    c = h = 0
    for f in itertools.permutations(range(V), qn):
        if any(lab[f[u]] != qlab[u] for u in range(qn)):
            continue
        if all((f[x], f[y]) in es for x, y in qedges):
            c += 1
            s = sum(fmix64((u << 32) | f[u]) for u in range(qn))
            h = (h + fmix64(F.HASH_SEED + s)) & M64
    return c, h


@pytest.mark.parametrize("seed", range(6))
def test_brute_force_count_and_hash(seed):
    rng = np.random.default_rng(seed)
    V = 11
    edges = [(i, j) for i in range(V) for j in range(i + 1, V) if rng.random() < 0.45]
    lab = rng.integers(0, 2, V).astype(np.int32)
    g = F.Graph(lab, np.asarray(edges, np.uint32).reshape(-1, 2))
    off, adj = g.csr()
    for qs in range(3):
        q = F.gen_query(g, 4, F.QUERY_INDUCED, seed=seed * 10 + qs, csr=(off, adj))
        qe = q.edges.tolist()
        c, h, lv = O.match(lab, off, adj, q.labels, q.edges)
        assert (c, h) == brute(V, edges, lab, 4, qe, q.labels.tolist())
        assert lv[-1] == c


def test_k4_plus_pendant_identity():
    """|K4+pendant| = sum over ordered K4 images of (deg(image of the attach vertex) - 3)."""
    rng = np.random.default_rng(3)
    V = 40
    edges = [(i, j) for i in range(V) for j in range(i + 1, V) if rng.random() < 0.3]
    off, adj = csr_of(V, edges)
    deg = np.diff(off.astype(np.int64))
    nb = [set(adj[off[v]:off[v + 1]].tolist()) for v in range(V)]
    expect = 0
    for f in itertools.permutations(range(V), 4):
        if all(f[j] in nb[f[i]] for i in range(4) for j in range(i + 1, 4)):
            expect += deg[f[0]] - 3
    q = complete(4) + [(0, 4)]
    assert count(V, edges, 5, q) == expect


def test_order_independence_of_count_and_hash():
    lab = F.gen_labels(1500, 6, "uniform", seed=9)
    g = F.gen_rmat(1500, 6000, seed=9, labels=lab)
    off, adj = g.csr()
    for s in range(4):
        q = F.gen_query(g, 6, F.QUERY_DENSE if s % 2 else F.QUERY_SPARSE, seed=s, csr=(off, adj))
        ref = O.match(g.labels, off, adj, q.labels, q.edges)
        rng = np.random.default_rng(s)
        # random connected orders
        for _ in range(3):
            n = q.num_vertices
            nbrs = {u: set() for u in range(n)}
            for a, b in q.edges.tolist():
                nbrs[a].add(b)
                nbrs[b].add(a)
            order = [int(rng.integers(n))]
            while len(order) < n:
                front = sorted({w for u in order for w in nbrs[u]} - set(order))
                order.append(int(rng.choice(front)))
            c, h, lv = O.match(g.labels, off, adj, q.labels, q.edges, order=order)
            assert (c, h) == ref[:2]
        assert ref[0] >= 1  # the source embedding exists


K4 = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


def test_k4_pendant_identity_counter():
    """The clique-listing counter (K4 subgraphs, and K4+pendant embeddings by
    6 * sum over K4s of sum of (deg - 3)) against the backtracking matcher, on
    complete graphs (closed form) and R-MAT graphs of the config-3 generator."""
    for n in (4, 5, 7):
        off, adj = csr_of(n, [(i, j) for i in range(n) for j in range(i + 1, n)])
        k4, pend = O.k4_pendant(off, adj)
        assert k4 == math.comb(n, 4)
        assert pend == math.perm(n, 5) if n >= 5 else pend == 0
    for s in (8, 9, 10):
        g = F.gen_rmat(1 << s, 1 << (s + 3), 0.57, 0.19, 0.19, seed=3)
        off, adj = g.csr()
        k4, pend = O.k4_pendant(off, adj)
        z = np.zeros(5, np.int32)
        assert 24 * k4 == O.match(g.labels, off, adj, z[:4], K4)[0]
        assert pend == O.match(g.labels, off, adj, z, K4 + [(0, 4)])[0]


def test_k4_pendant_counts_at_scale():
    """Recorded values at 2^12 and 2^16 vertices (16 edges per vertex, the
    config-3 density); the 2^12 count agrees with the engine's K4+pendant
    count on the same graph (1.02e11)."""
    want = {12: (10124699, 102446423832), 16: (454139239, 20214289911666)}
    for s, (k4, pend) in want.items():
        off, adj = F.gen_rmat(1 << s, 1 << (s + 4), 0.57, 0.19, 0.19, seed=3).csr()
        assert O.k4_pendant(off, adj) == (k4, pend)
