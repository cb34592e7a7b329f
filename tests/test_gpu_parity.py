"""GPU parity: the CUDA path through the C ABI against the oracle, bit-exact.

Transforms (device CSR, signature) are compared with the oracle restatements
that tests/test_oracle_pins.py pins to the reference; filters with the
restated GSI / MMatch filters and the refinement rule; counts and set hashes
with the oracle's backtracking matcher.
"""
import numpy as np
import pytest

import fsig_gb300 as F
from conftest import GOLDEN
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SIMPLE = ["small_l4", "mid_l8", "cl_zipf16", "unlabeled"]


def oracle_graph(name, golden):
    rec = golden["graphs"][name]
    return rec, O.read_tve(GOLDEN / rec["file"], rec["labeled"])


@pytest.mark.parametrize("name", SIMPLE + ["small_l4_trailing_newline"])
def test_device_csr_matches_reference_transform(engine, golden, name):
    rec, d = oracle_graph(name, golden)
    g = F.read_graph(GOLDEN / rec["file"], bool(rec["labeled"]))
    off, adj = engine.build_csr(d["V"], g.edges)
    assert np.array_equal(off, d["offsets"])
    assert np.array_equal(adj, d["edges"])


@pytest.mark.parametrize("name", SIMPLE)
@pytest.mark.parametrize("col", [0, 1])
def test_device_signature_matches_reference(engine, golden, name, col):
    rec, d = oracle_graph(name, golden)
    s = engine.build_signature(d["labels"], d["offsets"], d["edges"], col)
    assert np.array_equal(s, O.signature(d["labels"], d["offsets"], d["edges"], col))


def load_simple(engine, name, golden):
    rec, d = oracle_graph(name, golden)
    g = F.read_graph(GOLDEN / rec["file"], bool(rec["labeled"]))
    engine.load_graph(g)
    off, adj = O.simplify(d["offsets"], d["edges"])
    return g, d["labels"], off, adj


def golden_queries(golden, limit=None):
    qs = []
    for name, rec in sorted(golden["queries"].items()):
        qs.append(F.read_query(GOLDEN / rec["file"]))
    return qs[:limit] if limit else qs


def query_masks(q):
    n = q.num_vertices
    m = np.zeros(n, np.uint32)
    for a, b in q.edges.tolist():
        if a != b:
            m[a] |= 1 << b
            m[b] |= 1 << a
    return m


@pytest.mark.parametrize("classes", [True, False])
@pytest.mark.parametrize("refine", [0, 1, 3])
def test_filters_match_oracle(engine, golden, refine, classes):
    """Bit-exact flags.  With classes the members of a class share one
    bitmap, the thresholds are the class counts and dominated classes are
    tested first; the oracle has none of the sharing or early tests, only the
    rule, so equal flags show those change no outcome."""
    g, lab, off, adj = load_simple(engine, "cl_zipf16", golden)
    dsig = O.signature(lab, off, adj, 0)
    for q in golden_queries(golden):
        qoff, qadj = F.Graph(q.labels, q.edges).csr()
        qsig = O.signature(q.labels, qoff, qadj, 0).reshape(-1, 16)
        qdeg = np.diff(qoff.astype(np.int64))
        # GSI: label + signature subset (GSI_kernels.cuh:8-24), refinement optional
        gsi = np.stack([O.gsi_filter(dsig, qsig[u]) for u in range(q.num_vertices)])
        mm = np.stack([O.mmatch_init(lab, off, q.labels[u], qdeg[u]) for u in range(q.num_vertices)])
        fused = gsi & mm
        masks = query_masks(q)
        cls = O.refine_classes(q.labels, masks) if classes else None
        for algo, base in ((F.ALGO_GSI, gsi), (F.ALGO_FSIG, mm), (F.ALGO_FUSED, fused)):
            want = O.refine(lab, off, adj, masks, base, refine, cls) if refine else base
            got = engine.filter(q, algo, refine, classes=classes)
            assert np.array_equal(got, want), (algo, refine)


def match_oracle(lab, off, adj, q):
    return O.match(lab, off, adj, q.labels, q.edges)


@pytest.mark.parametrize("algo", [F.ALGO_FSIG, F.ALGO_GSI, F.ALGO_FUSED])
def test_golden_queries_count_and_hash(engine, golden, algo):
    """Against the oracle's results recorded with the fixtures (some golden
    queries have 10^8-10^9 embeddings, tens of seconds on the CPU); the cheap
    ones are also re-run live."""
    g, lab, off, adj = load_simple(engine, "cl_zipf16", golden)
    rec = golden["oracle_cl_zipf16"]
    for name in sorted(golden["queries"]):
        q = F.read_query(GOLDEN / golden["queries"][name]["file"])
        want = rec[name]
        if want["count"] < 2_000_000:
            assert match_oracle(lab, off, adj, q)[:2] == (want["count"], want["hash"])
        r = engine.match(q, algo)
        assert (r.count, r.hash) == (want["count"], want["hash"]), name
        assert r.level_counts[-1] == want["count"]
    rs = engine.match_batch(golden_queries(golden), algo=algo)
    assert [(r.count, r.hash) for r in rs] == [(rec[n]["count"], rec[n]["hash"]) for n in sorted(golden["queries"])]


@pytest.fixture(scope="module")
def config1():
    """R-MAT (a .57, b .19, c .19), seed 1, 10,000 vertices, 50,000 edges,
    8 uniform labels; 100 four-vertex random-walk queries."""
    lab = F.gen_labels(10000, 8, "uniform", seed=1)
    g = F.gen_rmat(10000, 50000, 0.57, 0.19, 0.19, seed=1, labels=lab)
    off, adj = g.csr()
    qs = [F.gen_query(g, 4, F.QUERY_INDUCED, seed=1000 + i, csr=(off, adj)) for i in range(100)]
    want = [match_oracle(g.labels, off, adj, q) for q in qs]
    return g, qs, want


@pytest.mark.parametrize("algo", [F.ALGO_FSIG, F.ALGO_GSI, F.ALGO_FUSED])
def test_config1_single_query_path(engine, config1, algo):
    g, qs, want = config1
    engine.load_graph(g)
    for q, (c, h, lv) in zip(qs, want):
        r = engine.match(q, algo)
        assert (r.count, r.hash) == (c, h)
        assert r.count >= 1


@pytest.mark.parametrize("algo", [F.ALGO_FSIG, F.ALGO_GSI, F.ALGO_FUSED])
def test_config1_batch(engine, config1, algo):
    g, qs, want = config1
    engine.load_graph(g)
    rs = engine.match_batch(qs, algo=algo)
    for r, (c, h, lv) in zip(rs, want):
        assert r.status == 0
        assert (r.count, r.hash) == (c, h)


def test_given_orders_and_level_counts(engine, config1):
    g, qs, want = config1
    engine.load_graph(g)
    off, adj = g.csr()
    for q, (c, h, lv) in list(zip(qs, want))[:20]:
        base = engine.match(q, F.ALGO_GSI)
        order = list(reversed(base.order))
        # reversed order is connected only sometimes; fall back to the plan order
        nb = {u: set() for u in range(q.num_vertices)}
        for a, b in q.edges.tolist():
            nb[a].add(b)
            nb[b].add(a)
        if not all(nb[order[k]] & set(order[:k]) for k in range(1, len(order))):
            order = base.order
        q2 = F.Query(q.labels, q.edges, order=np.asarray(order, np.uint32))
        r = engine.match_batch([q2], algo=F.ALGO_FUSED, order_source=F.ORDER_GIVEN)[0]
        assert (r.count, r.hash) == (c, h)
        assert r.order == order
        # Partial-embedding counts per depth depend on the filter; with the
        # label+degree filter alone they equal the oracle's, depth by depth.
        r0 = engine.match_batch([q2], algo=F.ALGO_FSIG, order_source=F.ORDER_GIVEN, refine_iters=0)[0]
        oc = O.match(g.labels, off, adj, q.labels, q.edges, order=order)
        assert r0.level_counts == [int(x) for x in oc[2]]
        assert all(a <= b for a, b in zip(r.level_counts, r0.level_counts))


def test_edge_cases(engine):
    lab = np.array([0, 1, 0, 1, 2, 0, 0], np.int32)
    edges = np.array([[0, 1], [1, 2], [2, 3], [3, 0], [0, 2], [4, 4], [1, 2], [5, 6]], np.uint32)
    g = F.Graph(lab, edges)
    engine.load_graph(g)
    off, adj = g.csr()  # simple graph: duplicate (1,2) and loop (4,4) collapse
    cases = [
        F.Query(np.array([0], np.int32), np.zeros((0, 2), np.uint32)),           # one vertex
        F.Query(np.array([2], np.int32), np.zeros((0, 2), np.uint32)),           # isolated data vertex
        F.Query(np.array([0, 1], np.int32), np.array([[0, 1]], np.uint32)),
        F.Query(np.array([0, 0], np.int32), np.array([[0, 1]], np.uint32)),
        F.Query(np.array([0, 1, 0], np.int32), np.array([[0, 1], [1, 2], [0, 2]], np.uint32)),
        F.Query(np.array([0, 1, 0, 1], np.int32), np.array([[0, 1], [1, 2], [2, 3], [3, 0]], np.uint32)),
        F.Query(np.array([2, 0], np.int32), np.array([[0, 1]], np.uint32)),     # no candidates
        F.Query(np.array([7, 0], np.int32), np.array([[0, 1]], np.uint32)),     # label absent from the graph
        F.Query(np.array([0, 1], np.int32), np.array([[0, 1], [0, 1], [1, 1]], np.uint32)),  # dup + self-loop
    ]
    for q in cases:
        c, h, lv = O.match(lab, off, adj, q.labels, q.edges)
        for algo in (F.ALGO_FSIG, F.ALGO_GSI, F.ALGO_FUSED):
            r = engine.match(q, algo)
            assert (r.count, r.hash) == (c, h), (q, algo)
        rb = engine.match_batch(cases)
        assert [(r.count, r.hash) for r in rb] == [
            tuple(O.match(lab, off, adj, x.labels, x.edges)[:2]) for x in cases]
    with pytest.raises(F.FsigError) as ei:
        engine.match(F.Query(np.array([0, 0, 0], np.int32), np.array([[0, 1]], np.uint32)))
    assert ei.value.status == F.EQUERY
    r = engine.match_batch([F.Query(np.array([0, 0, 0], np.int32), np.array([[0, 1]], np.uint32)), cases[2]])
    assert r[0].status == F.EQUERY and r[1].status == 0


def test_load_graph_file_reference_semantics(engine, golden, tmp_path):
    rec, d = oracle_graph("small_l4_trailing_newline", golden)
    engine.load_graph_file(GOLDEN / rec["file"], True)
    info = engine.graph_info()
    off, adj = O.simplify(d["offsets"], d["edges"])
    assert info["V"] == d["V"] and info["adj"] == len(adj)
    q = F.Query(np.array([0, 1, 2], np.int32), np.array([[0, 1], [1, 2]], np.uint32))
    c, h, _ = O.match(d["labels"], off, adj, q.labels, q.edges)
    r = engine.match(q, F.ALGO_GSI)
    assert (r.count, r.hash) == (c, h)
    engine.load_graph_file(GOLDEN / rec["file"], False)  # graph_type 0: every label 0
    q0 = F.Query(np.zeros(3, np.int32), q.edges)
    c0, h0, _ = O.match(np.zeros(d["V"], np.int32), off, adj, q0.labels, q0.edges)
    assert (engine.match(q0, F.ALGO_FSIG).count, engine.match(q0, F.ALGO_FSIG).hash) == (c0, h0)


def test_vertex_count_not_multiple_of_32_and_isolated(engine):
    for V in (1, 31, 33, 1000, 4097):
        rng = np.random.default_rng(V)
        lab = rng.integers(0, 3, V).astype(np.int32)
        E = min(V * 2, V * (V - 1) // 2)
        edges = rng.integers(0, V, (E, 2)).astype(np.uint32) if V > 1 else np.zeros((0, 2), np.uint32)
        g = F.Graph(lab, edges)
        engine.load_graph(g)
        off, adj = g.csr()
        for q in (F.Query(np.array([1], np.int32), np.zeros((0, 2), np.uint32)),
                  F.Query(np.array([0, 1, 2], np.int32), np.array([[0, 1], [1, 2]], np.uint32))):
            c, h, _ = O.match(lab, off, adj, q.labels, q.edges)
            r = engine.match(q, F.ALGO_FUSED)
            assert (r.count, r.hash) == (c, h)


@pytest.fixture(scope="module")
def config2_small():
    """The config-2 generator (Chung-Lu, exponent 2.1, 16 Zipf labels) at a
    tenth of its size, with dense and sparse 8-vertex queries."""
    lab = F.gen_labels(32000, 16, "zipf", seed=2)
    g = F.gen_chung_lu(32000, 105000, 2.1, seed=2, labels=lab)
    off, adj = g.csr()
    qs = []
    for i in range(24):
        mode = F.QUERY_DENSE if i % 2 == 0 else F.QUERY_SPARSE
        qs.append(F.gen_query(g, 8, mode, seed=2000 + i, csr=(off, adj)))
    # keep the suite fast: queries of at most 2e8 embeddings (found on the GPU)
    from fsig_gb300 import Engine
    with Engine(0, arena_bytes=4 << 30) as e:
        e.load_graph(g)
        counts = [r.count for r in e.match_batch(qs)]
    qs = [q for q, c in zip(qs, counts) if c <= 200_000_000]
    assert len(qs) >= 16
    return g, off, adj, qs


def test_config2_small_vs_oracle(engine, config2_small):
    g, off, adj, qs = config2_small
    engine.load_graph(g)
    rs = engine.match_batch(qs, algo=F.ALGO_FUSED)
    checked = 0
    for q, r in zip(qs, rs):
        assert r.status == 0
        # the oracle checks the ones it finishes quickly; all are checked for
        # agreement across algorithms below
        if r.count <= 20_000_000:
            c, h, _ = O.match(g.labels, off, adj, q.labels, q.edges)
            assert (r.count, r.hash) == (c, h)
            checked += 1
    assert checked >= 12


def test_algorithms_agree_at_scale(engine, config2_small):
    """Size-independent property: FSIG, GSI, fused and batched paths return
    the same count and set hash for every query, however large."""
    g, off, adj, qs = config2_small
    engine.load_graph(g)
    b = engine.match_batch(qs, algo=F.ALGO_GSI)
    for q, rb in zip(qs, b):
        r1 = engine.match(q, F.ALGO_FSIG)
        r3 = engine.match(q, F.ALGO_FUSED)
        assert (r1.count, r1.hash) == (rb.count, rb.hash) == (r3.count, r3.hash)


def test_work_splitting_preserves_results(engine, config2_small):
    """Forcing the frontier hand-off on almost every task (tiny cycle budget,
    short ranges, one task per grab) changes how the work is cut, never the
    count, the hash or the per-depth counts."""
    g, off, adj, qs = config2_small
    engine.load_graph(g)
    base = engine.match_batch(qs, algo=F.ALGO_FUSED)
    for kw in (dict(split_cycles=2000, split_len=32, chunk=1), dict(split_cycles=20000, split_len=64, chunk=2)):
        r = engine.match_batch(qs, algo=F.ALGO_FUSED, **kw)
        assert [(x.count, x.hash, x.level_counts) for x in r] == [(x.count, x.hash, x.level_counts) for x in base]
    single = [engine.match_batch([q], algo=F.ALGO_FUSED, split_cycles=2000, split_len=32)[0] for q in qs[:6]]
    assert [(x.count, x.hash) for x in single] == [(x.count, x.hash) for x in base[:6]]


@pytest.mark.parametrize("algo", [F.ALGO_FSIG, F.ALGO_GSI, F.ALGO_FUSED])
def test_refinement_classes_change_no_result(engine, config2_small, golden, algo):
    """Refinement with classes (shared bitmaps, class thresholds, dominated
    classes tested first) against per-vertex refinement: the same count and
    hash for every query, never more candidates, and the class thresholds
    prune somewhere."""
    g, off, adj, qs = config2_small
    engine.load_graph(g)
    fewer = 0
    for refine in (-1, 3):
        on = engine.match_batch(qs, algo=algo, refine_iters=refine)
        off_ = engine.match_batch(qs, algo=algo, refine_iters=refine, classes=False)
        for a, b, q in zip(on, off_, qs):
            assert (a.count, a.hash) == (b.count, b.hash)
            n = q.num_vertices
            assert all(x <= y for x, y in zip(a.candidates[:n], b.candidates[:n]))
            fewer += sum(a.candidates[:n]) < sum(b.candidates[:n])
    sym = [F.Query(np.zeros(k, np.int32), np.array([(i, (i + 1) % k) for i in range(k)], np.uint32))
           for k in (4, 5, 6)]
    sym.append(F.Query(np.array([0, 1, 1, 1, 1], np.int32), np.array([(0, i) for i in range(1, 5)], np.uint32)))
    gl, lab, offs, adjs = load_simple(engine, "cl_zipf16", golden)
    for q in sym + golden_queries(golden, 8):
        a = engine.match_batch([q], algo=algo, refine_iters=3)[0]
        b = engine.match_batch([q], algo=algo, refine_iters=3, classes=False)[0]
        assert (a.count, a.hash) == (b.count, b.hash)
        n = q.num_vertices
        assert all(x <= y for x, y in zip(a.candidates[:n], b.candidates[:n]))
        fewer += sum(a.candidates[:n]) < sum(b.candidates[:n])
        if a.count <= 2_000_000:
            c, h, _ = O.match(lab, offs, adjs, q.labels, q.edges)
            assert (a.count, a.hash) == (c, h)
    assert fewer > 0


@pytest.mark.parametrize("algo", [F.ALGO_FSIG, F.ALGO_GSI, F.ALGO_FUSED])
def test_cuda_graph_batches_match_stream_batches(engine, config2_small, algo):
    """A batch run as one CUDA graph (replayed with updated parameters batch
    after batch) returns what the same batch returns as ordinary launches,
    including when records overflow into further passes after the graph."""
    g, off, adj, qs = config2_small
    engine.load_graph(g)
    base = engine.match_batch(qs, algo=algo)
    assert engine.last_stats()["graph"] == 0
    want = [(x.count, x.hash, x.level_counts, x.order) for x in base]
    for kw in (dict(), dict(split_cycles=2000, split_len=32, chunk=1)):
        for part in (qs, qs[: len(qs) // 2], qs):  # different shapes, then the first again
            r = engine.match_batch(part, algo=algo, use_graph=True, **kw)
            assert engine.last_stats()["graph"] == 1
            assert [(x.count, x.hash, x.level_counts, x.order) for x in r] == want[: len(part)]


def test_graph_cache_round_trip(engine, golden, tmp_path):
    """A graph store saved to the binary cache and loaded into another engine
    matches every golden query exactly as the built one does."""
    rec = golden["graphs"]["cl_zipf16"]
    engine.load_graph(F.read_graph(GOLDEN / rec["file"], True))
    qs = golden_queries(golden)
    want = [(r.count, r.hash, r.order) for r in engine.match_batch(qs, algo=F.ALGO_FUSED)]
    info = engine.graph_info()
    path = tmp_path / "cl_zipf16.fsigcache"
    engine.save_graph_cache(path)
    with F.Engine(0, arena_bytes=1 << 30) as other:
        other.load_graph_cache(path)
        assert other.graph_info() == info
        got = [(r.count, r.hash, r.order) for r in other.match_batch(qs, algo=F.ALGO_FUSED)]
        assert got == want
        assert [(r.count, r.hash) for r in (other.match(q, F.ALGO_FSIG) for q in qs[:4])] == [w[:2] for w in want[:4]]
    (tmp_path / "bad.fsigcache").write_bytes(b"not a cache")
    with pytest.raises(F.FsigError) as ei:
        engine.load_graph_cache(tmp_path / "bad.fsigcache")
    assert ei.value.status == F.EIO


@pytest.mark.parametrize("name", ["small_l4", "small_l4_trailing_newline", "mid_l8", "cl_zipf16"])
def test_device_pcsr_matches_reference(engine, golden, name):
    """The PCSR units built on the device equal the reference's own output
    (recorded digests) and the oracle's restatement word for word."""
    import hashlib
    rec, d = oracle_graph(name, golden)
    units = engine.build_pcsr(d["labels"], d["offsets"], d["edges"], d["L"])
    assert len(units) == rec["pcsr_units"]

    def sha(a):
        return hashlib.sha256(np.ascontiguousarray(a, np.uint32).tobytes()).hexdigest()

    for (k, m, off, e), (rk, rm, roff, re_) in zip(units, rec["pcsr"]):
        assert (k, m) == (rk, rm)
        assert sha(off) == roff and sha(e) == re_
    for (k, m, off, e), (ok, om, ooff, oe) in zip(units, O.pcsr(d["labels"], d["offsets"], d["edges"], d["L"])):
        assert (k, m) == (ok, om) and np.array_equal(off, ooff) and np.array_equal(e, oe)


def test_device_pcsr_with_overflow_chains(engine):
    """A unit whose bucket gets more than 15 keys, so that its slot chains to
    the first empty bucket: a star whose 20 leaves all hash to bucket 3 of the
    unit's 21 keys."""
    nk = 21
    leaves = [v for v in range(1, 5000) if O.murmur2_u32(v) % nk == 3][:20]
    lab = np.zeros(max(leaves) + 1, np.int32)
    lab[leaves] = 1
    g = F.Graph(lab, np.array([(0, v) for v in leaves], np.uint32))
    off, adj = g.csr()
    ref = O.pcsr(lab, off, adj, 2)
    assert (ref[0][2].reshape(-1, 32)[:, 30] != 0xFFFFFFFF).sum() == 1  # one chained slot
    units = engine.build_pcsr(lab, off, adj, 2)
    for (k, m, o, e), (ok, om, ooff, oe) in zip(units, ref):
        assert (k, m) == (ok, om) and np.array_equal(o, ooff) and np.array_equal(e, oe)
