"""Refinement classes and the class-count refinement rule, on the CPU.

The classes (fsig_refine_classes, host code of the engine) against the
oracle's own colour refinement, their defining properties, their relation to
the reference's MMatch::find_equivalent_classes (match/MMatch.cu:44-173,
recorded in the golden fixtures), the dominated classes, and the oracle's
refinement rule: stronger than the per-vertex rule and never dropping the
image of an embedding (brute force on small graphs)."""

import numpy as np
import pytest

import fsig_gb300 as F
import oracle.oracle as O
from conftest import GOLDEN


def masks_of(q):
    n = q.num_vertices
    m = np.zeros(n, np.uint32)
    for a, b in q.edges.tolist():
        if a != b:
            m[a] |= 1 << b
            m[b] |= 1 << a
    return m


def sym_queries():
    """Queries with non-trivial classes: cycles, stars, complete and
    complete bipartite graphs, a prism, a path, with one or two labels."""
    out = []

    def q(labels, edges):
        out.append(F.Query(np.array(labels, np.int32), np.array(edges, np.uint32).reshape(-1, 2)))

    for n in (3, 4, 5, 6, 8):
        q([0] * n, [(i, (i + 1) % n) for i in range(n)])
        q([i % 2 for i in range(n)], [(i, (i + 1) % n) for i in range(n)])
        q([0] + [1] * (n - 1), [(0, i) for i in range(1, n)])
        q([0] * n, [(i, j) for i in range(n) for j in range(i + 1, n)])
        q([0] * n, [(i, i + 1) for i in range(n - 1)])
    q([0, 0, 1, 1, 1], [(a, b) for a in (0, 1) for b in (2, 3, 4)])
    q([0] * 6, [(0, 1), (1, 2), (2, 0), (3, 4), (4, 5), (5, 3), (0, 3), (1, 4), (2, 5)])
    q([0, 0, 0, 0, 1], [(0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (2, 4)])
    return out


def random_queries(seed, count, n_lo=3, n_hi=12, labels=3):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count:
        n = int(rng.integers(n_lo, n_hi + 1))
        edges = {(i, int(rng.integers(0, i))) for i in range(1, n)}  # a random tree, then chords
        for _ in range(int(rng.integers(0, n))):
            a, b = (int(x) for x in rng.integers(0, n, 2))
            if a != b:
                edges.add((max(a, b), min(a, b)))
        out.append(F.Query(rng.integers(0, labels, n).astype(np.int32), np.array(sorted(edges), np.uint32)))
    return out


def all_queries(golden):
    qs = [F.read_query(GOLDEN / rec["file"]) for _, rec in sorted(golden["queries"].items())]
    return qs + sym_queries() + random_queries(7, 200)


def test_classes_match_oracle(golden):
    for q in all_queries(golden):
        got = F.refine_classes(q)["classes"]
        assert got == O.refine_classes(q.labels, masks_of(q)), q.edges.tolist()


def test_classes_are_equitable(golden):
    for q in all_queries(golden):
        m = masks_of(q)
        n = q.num_vertices
        sig = O.query_signature(q.labels, m)
        cls = F.refine_classes(q)["classes"]
        reps = sorted(set(cls))

        def counts(u):
            return [sum(1 for w in range(n) if (int(m[u]) >> w) & 1 and cls[w] == r) for r in reps]

        for u in range(n):
            r = cls[u]
            assert r <= u and cls[r] == r
            assert q.labels[u] == q.labels[r] and np.array_equal(sig[u], sig[r])
            assert counts(u) == counts(r)


def test_classes_coarser_than_reference(golden):
    """Vertices the reference puts in one class share one here as well (the
    reference's classes meet the same conditions, with a degree cut-off on its
    permutation search that can only split more)."""
    seen = 0
    for name, rec in sorted(golden["queries"].items()):
        q = F.read_query(GOLDEN / rec["file"])
        ours = F.refine_classes(q)["classes"]
        ref = rec["cases"][0]["mm_classes"]
        for u in range(q.num_vertices):
            for v in range(q.num_vertices):
                if ref[u] == ref[v]:
                    assert ours[u] == ours[v], (name, u, v)
                    seen += u != v
    assert seen > 0


def test_symmetric_queries_collapse():
    # one class for a labelled cycle and a clique; centre + leaves for a star
    qs = sym_queries()
    c6 = F.Query(np.zeros(6, np.int32), np.array([(i, (i + 1) % 6) for i in range(6)], np.uint32))
    assert F.refine_classes(c6)["classes"] == [0] * 6
    star = F.Query(np.array([0, 1, 1, 1], np.int32), np.array([(0, 1), (0, 2), (0, 3)], np.uint32))
    assert F.refine_classes(star)["classes"] == [0, 1, 1, 1]
    path = F.Query(np.zeros(5, np.int32), np.array([(i, i + 1) for i in range(4)], np.uint32))
    assert F.refine_classes(path)["classes"] == [0, 1, 2, 1, 0]
    assert len(qs) > 20


def test_dominated_classes_are_implied(golden):
    found = 0
    for q in all_queries(golden):
        m = masks_of(q)
        n = q.num_vertices
        sig = O.query_signature(q.labels, m)
        rc = F.refine_classes(q)
        cls, dom = rc["classes"], rc["dominated"]
        reps = sorted(set(cls))

        def counts(u):
            return [sum(1 for w in range(n) if (int(m[u]) >> w) & 1 and cls[w] == r) for r in reps]

        for u in range(n):
            d = dom[u]
            if cls[u] != u:
                assert d == F.NO_CLASS
                continue
            if d == F.NO_CLASS:
                continue
            found += 1
            assert cls[d] == d and d != u and q.labels[d] == q.labels[u]
            assert bin(int(m[d])).count("1") <= bin(int(m[u])).count("1")
            assert all((int(a) & ~int(b)) == 0 for a, b in zip(sig[d][1:], sig[u][1:]))
            assert all(a <= b for a, b in zip(counts(d), counts(u)))
    assert found > 10


# ---------------------------------------------------------------------------
# the rule, on small data graphs
# ---------------------------------------------------------------------------
def small_graph(seed, V=40, deg=4, labels=2):
    rng = np.random.default_rng(seed)
    edges = set()
    while len(edges) < V * deg // 2:
        a, b = (int(x) for x in rng.integers(0, V, 2))
        if a != b:
            edges.add((min(a, b), max(a, b)))
    lab = rng.integers(0, labels, V).astype(np.int32)
    e = np.array(sorted(edges), np.uint32)
    off, adj = F.Graph(lab, e).csr()
    return lab, np.asarray(off, np.uint32), np.asarray(adj, np.uint32)


def base_flags(lab, off, adj, q):
    m = masks_of(q)
    deg = [bin(int(x)).count("1") for x in m]
    return np.stack([O.mmatch_init(lab, off, q.labels[u], deg[u]) for u in range(q.num_vertices)])


def embeddings(lab, off, adj, q):
    """All embeddings (tuples of data vertices), by plain backtracking."""
    n = q.num_vertices
    nb = [set(adj[off[v]:off[v + 1]].tolist()) for v in range(len(lab))]
    qn = [[w for w in range(n) if (int(masks_of(q)[u]) >> w) & 1] for u in range(n)]
    out = []

    def go(f):
        u = len(f)
        if u == n:
            out.append(tuple(f))
            return
        for v in range(len(lab)):
            if lab[v] != q.labels[u] or v in f:
                continue
            if all(f[w] in nb[v] for w in qn[u] if w < u):
                go(f + [v])

    go([])
    return out


def small_queries():
    qs = [q for q in sym_queries() if q.num_vertices <= 5]
    qs += random_queries(11, 30, 3, 5, labels=2)
    return qs


@pytest.mark.parametrize("seed", [1, 2])
def test_class_rule_is_sound_and_stronger(seed):
    lab, off, adj = small_graph(seed)
    pruned = 0
    for q in small_queries():
        m = masks_of(q)
        base = base_flags(lab, off, adj, q)
        cls = O.refine_classes(q.labels, m)
        for it in (1, 3):
            plain = O.refine(lab, off, adj, m, base, it)
            strong = O.refine(lab, off, adj, m, base, it, cls)
            assert np.all(strong <= plain)
            pruned += int(plain.sum() - strong.sum())
            for f in embeddings(lab, off, adj, q):
                for u, v in enumerate(f):
                    assert strong[u, v], (q.edges.tolist(), f)
    assert pruned > 0


def test_dominated_candidate_sets_nest():
    """C(u) within C(dom[u]) after every refinement step, the fact the early
    test in the refinement kernel rests on."""
    lab, off, adj = small_graph(3, V=60, deg=5, labels=2)
    nested = 0
    for q in small_queries() + random_queries(5, 40, 4, 8, labels=2):
        m = masks_of(q)
        rc = F.refine_classes(q)
        base = base_flags(lab, off, adj, q)
        for it in range(4):
            c = O.refine(lab, off, adj, m, base, it, rc["classes"]) if it else base
            for u, d in enumerate(rc["dominated"]):
                if d != F.NO_CLASS:
                    assert np.all(c[u] <= c[d]), (q.edges.tolist(), u, d, it)
                    nested += 1
    assert nested > 0


def test_class_members_keep_equal_flags():
    lab, off, adj = small_graph(4, V=60, deg=5, labels=2)
    for q in small_queries():
        m = masks_of(q)
        cls = O.refine_classes(q.labels, m)
        c = O.refine(lab, off, adj, m, base_flags(lab, off, adj, q), 3, cls)
        for u in range(q.num_vertices):
            assert np.array_equal(c[u], c[cls[u]])
