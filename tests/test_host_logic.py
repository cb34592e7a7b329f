"""Host-side logic of the learned order, the autotuner and the bench's
fallback feed, against fake engines (no GPU)."""
import numpy as np
import pytest

import fsig_gb300 as F
from fsig_gb300 import autotune, learn


class FakeResult:
    def __init__(self, count, hash_, status=0, work=0, candidates=None, order=None):
        self.count, self.hash, self.status, self.work = count, hash_, status, work
        self.candidates = candidates or []
        self.order = order or []
        self.level_counts = []


def query(n, extra=()):
    edges = [(i, i + 1) for i in range(n - 1)] + list(extra)
    return F.Query(np.zeros(n, np.int32), np.asarray(edges, np.uint32))


class KnobEngine:
    """Device time depends on the knobs; results never do (unless broken)."""

    def __init__(self, broken=None):
        self.broken = broken
        self.ms = 0.0

    def match_batch(self, qs, **kw):
        self.ms = 10.0 + abs(kw.get("chunk", 1) - 2) + abs(kw.get("split_len", 256) - 512) / 256 \
            + (0 if kw.get("warps_per_block", 8) == 8 else 1) + abs(kw.get("split_cycles", 4000) - 16000) / 16000 \
            + 0.5 * abs(kw.get("isect", 0) - 1) + (0.25 if kw.get("refine_coop", 32) != 128 else 0)
        bad = self.broken is not None and kw.get("chunk") == self.broken
        return [FakeResult(i + (1 if bad else 0), 7 * i) for i, _ in enumerate(qs)]

    def last_stats(self):
        return {"ms_filter": 0.0, "ms_join": self.ms}


def test_autotune_finds_the_fastest_setting():
    best, trials = autotune.tune(KnobEngine(), [query(3)] * 4, repeats=1)
    assert best == {"warps_per_block": 8, "chunk": 2, "split_len": 512, "split_cycles": 16000, "isect": 1}
    assert trials[0][0] == autotune.DEFAULTS
    # the refinement's warps-per-candidate split joins when the batch refines
    best, _ = autotune.tune(KnobEngine(), [query(3)] * 4, repeats=1, refine_iters=1)
    assert best == {"warps_per_block": 8, "chunk": 2, "split_len": 512, "split_cycles": 16000, "isect": 1,
                    "refine_coop": 128}


class WindowEngine(KnobEngine):
    """Learned order: the window changes device time and which queries go
    over the work limit (status ELIMIT, no result); heuristic runs cost 3 ms
    per query."""
    BATCH_MS = {1: 10.5, 2: 10.2, 4: 10.8, 32: 9.0}

    def match_batch(self, qs, **kw):
        super().match_batch(qs, **kw)
        if kw["order_source"] == F.ORDER_HEURISTIC:
            self.ms = 3.0 * len(qs)
            return [FakeResult(int(q.labels.size) * 100, 7) for q in qs]
        w = kw["learned_window"]
        self.ms += self.BATCH_MS[w] - 10.0
        over = 2 if w == 32 else 0
        return [FakeResult(0, 0, F.ELIMIT) if i < over else FakeResult(int(q.labels.size) * 100, 7)
                for i, q in enumerate(qs)]


def test_autotune_learned_window_counts_the_fallback_runs():
    qs = [query(3 + i) for i in range(4)]
    best, trials = autotune.tune(WindowEngine(), qs, order_source=F.ORDER_LEARNED, repeats=1)
    # window 32 is fastest per batch, but its two fallbacks cost 6 ms more
    assert best["learned_window"] == 2
    assert best["chunk"] == 2 and best["split_len"] == 512
    assert trials[0][0] == {**autotune.DEFAULTS, **autotune.LEARNED_DEFAULTS}
    plain, _ = autotune.tune(KnobEngine(), qs, repeats=1)
    assert "learned_window" not in plain


def test_autotune_rejects_a_setting_that_changes_results():
    with pytest.raises(RuntimeError):
        autotune.tune(KnobEngine(broken=8), [query(3)] * 4, repeats=1)


@pytest.mark.parametrize("n", [2, 5, 9, 16])
def test_alternative_orders_are_distinct_connected_permutations(n):
    q = query(n, extra=[(0, n - 1)] if n > 2 else [])
    masks = learn.adjacency_masks(q)
    rng = np.random.default_rng(n)
    heur = list(range(n))
    alts = learn.alternative_orders(q, list(range(1, n + 1)), 12, rng, around=heur)
    assert len({tuple(o) for o in alts}) == len(alts)
    assert heur not in alts
    for o in alts:
        assert sorted(o) == heur and learn.is_connected_order(o, masks)


def test_best_order_needs_the_margin():
    lg = learn.QueryLog(query(3), [1, 1, 1], 5, 9, [0, 1, 2], 100, [[1, 0, 2], [2, 1, 0]], [99, 97], [], 0)
    assert lg.best == ([2, 1, 0], 97)           # 97 < 0.98 x 100
    lg.works = [99, 98.5]
    assert lg.best == ([0, 1, 2], 100)          # neither is 2% cheaper
    lg.works = [99, 97]
    lg.margin = 0.9
    assert lg.best == ([0, 1, 2], 100)          # 97 is not 10% cheaper


def test_training_targets_are_positions_of_the_best_order():
    class FeatEngine:
        def mpnn_features(self, qs, cands, algo):
            return np.zeros((sum(q.num_vertices for q in qs), 8), np.float32)
    logs = [learn.QueryLog(query(3), [1, 1, 1], 1, 1, [0, 1, 2], 10, [[2, 1, 0]], [1], [], 0),
            learn.QueryLog(query(2), [1, 1], 1, 1, [0, 1], 10, [], [], [], 0)]
    goff, feat, nbr, tgt = learn.training_set(FeatEngine(), logs)
    assert list(goff) == [0, 3, 5]
    assert list(tgt) == [1.0, 0.5, 0.0, 0.0, 1.0]
    assert list(nbr[:3]) == [0b010, 0b101, 0b010]


class FeedEngine:
    """A learned batch puts query 'x' over the limit; given orders are kept."""

    def __init__(self):
        self.calls = []

    def match_batch(self, qs, **kw):
        self.calls.append([q.order is not None for q in qs])
        out = []
        for q in qs:
            tag = int(q.labels[0])
            if tag == 99 and q.order is None:
                out.append(FakeResult(0, 0, status=F.ELIMIT, candidates=[3, 2, 1]))
            else:
                out.append(FakeResult(tag, tag * 10))
        return out

    def last_stats(self):
        return {"ms_filter": 0.0, "ms_join": 1.0, "ms_enum": 1.0, "enum_bytes": 0, "kernel_launches": 1,
                "enum_passes": 1, "h2d_bytes": 0, "d2h_bytes": 0}


def test_fallbacks_ride_along_in_the_next_batch(monkeypatch):
    monkeypatch.setattr(F, "plan_order", lambda q, algo, cand: {"order": [2, 1, 0]})
    eng = FeedEngine()
    feed = learn.LearnedFeed(eng, F.ALGO_FUSED, 1 << 20)
    stats = []

    def q(tag):
        return F.Query(np.full(3, tag, np.int32), np.asarray([(0, 1), (1, 2)], np.uint32))

    batches = [[q(1), q(99)], [q(2), q(3)]]
    results = [None, None]
    _, fb0 = feed.step(0, batches[0], results, stats.append)
    _, fb1 = feed.step(1, batches[1], results, stats.append)
    feed.flush(results, stats.append)
    assert (fb0, fb1) == (1, 0)
    assert eng.calls == [[False, False], [False, False, True]]  # the fallback rides in batch 1 with its order
    assert results == [[(1, 10), (99, 990)], [(2, 20), (3, 30)]]
    assert len(stats) == 2


def test_batch_packing_matches_per_query_packing():
    """The vectorized fsig_query array of a batch points at the same labels,
    edges and orders as packing each query on its own."""
    rng = np.random.default_rng(4)
    qs = []
    for i in range(40):
        n = int(rng.integers(1, 33))
        e = [(j, int(rng.integers(0, j))) for j in range(1, n)]
        q = F.Query(rng.integers(0, 5, n).astype(np.int32), np.asarray(e, np.uint32).reshape(-1, 2))
        if i % 3 == 0:
            q = F.Query(q.labels, q.edges, order=np.arange(n, dtype=np.uint32))
        qs.append(q)
    ptr, keep = F._pack_queries(qs)
    for i, q in enumerate(qs):
        a = ptr[i]
        assert (a.num_vertices, a.num_edges) == (q.num_vertices, len(q.edges))
        assert list(a.labels[:a.num_vertices]) == q.labels.tolist()
        assert list(a.edges[:2 * a.num_edges]) == np.asarray(q.edges).reshape(-1).tolist()
        assert bool(a.order) == (q.order is not None)
        if q.order is not None:
            assert list(a.order[:a.num_vertices]) == q.order.tolist()


def test_batch_packing_refuses_an_order_of_the_wrong_length():
    """Each order pointer is placed by its query's vertex count, so an order
    of another length would shift every later query's: refused up front."""
    q = F.Query(np.zeros(3, np.int32), np.array([[0, 1], [1, 2]], np.uint32))
    bad = F.Query(q.labels, q.edges, order=np.arange(2, dtype=np.uint32))
    with pytest.raises(ValueError):
        F._pack_queries([q, bad, q])
    F._pack_queries([q, F.Query(q.labels, q.edges, order=np.arange(3, dtype=np.uint32))])
