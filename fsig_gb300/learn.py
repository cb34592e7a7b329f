"""Learned matching order: parameters of the order-scoring network, the
order/cost logs the engine produces, and training with the engine's own
forward and backward kernels (``fsig_mpnn_train_step``).

The reference has no counterpart: it orders by heuristics only
(match/GSI.cu:105-149, match/MMatch.cu:1575-1641).  Here the heuristic order
stays the fallback and the measure of cost:

* a log records, per query, the heuristic order and a set of alternative
  connected orders, each with the driver entries its enumeration examined
  (``work``, deterministic) and its per-level intermediate counts;
  alternatives run under a work limit equal to the heuristic's own work, so an
  alternative that is not better stops early and a log costs at most
  (alternatives + 1) heuristic runs;
* the network sees the heuristic order (each vertex's position in it) among
  its inputs, so it learns corrections to that order;
* the training target of a vertex is its position in the cheapest order found,
  divided by n - 1; the batched path orders by lowest score among the
  frontier, so a network that fits the targets reproduces that order;
* at serving time a learned-order query that exceeds its work limit is run
  again with the heuristic order, so counts never depend on the network.
"""
from __future__ import annotations

import dataclasses
from pathlib import Path
from typing import Sequence

import numpy as np

from . import (ALGO_FUSED, ELIMIT, ORDER_GIVEN, ORDER_HEURISTIC, ORDER_LEARNED, Engine, Query,
               mpnn_param_count)

F_IN, F_PAD, H, LAYERS = 8, 16, 64, 3
P_WIN = 0
P_BIN = P_WIN + F_PAD * H
P_WS = P_BIN + H
P_WN = P_WS + LAYERS * H * H
P_B = P_WN + LAYERS * H * H
P_WOUT = P_B + LAYERS * H
P_BOUT = P_WOUT + H
N_PARAMS = P_BOUT + 1

WEIGHTS = Path(__file__).resolve().parent / "order_net.npy"
UNCAPPED = 1 << 60  # a work limit that only turns on counting


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights, zero biases; the padding rows of W_in stay zero."""
    assert N_PARAMS == mpnn_param_count()
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, np.float32)
    w_in = np.zeros((F_PAD, H), np.float32)
    w_in[:F_IN] = rng.normal(0, np.sqrt(2.0 / F_IN), (F_IN, H))
    p[P_WIN:P_BIN] = w_in.reshape(-1)
    p[P_WS:P_WN] = rng.normal(0, np.sqrt(1.0 / H), LAYERS * H * H)
    p[P_WN:P_B] = rng.normal(0, np.sqrt(1.0 / H), LAYERS * H * H)
    p[P_WOUT:P_BOUT] = rng.normal(0, np.sqrt(1.0 / H), H)
    p[P_BOUT] = 0.5
    return p


def load_params(path=None) -> np.ndarray:
    p = np.load(path or WEIGHTS).astype(np.float32)
    if p.size != N_PARAMS:
        raise ValueError(f"{path}: {p.size} parameters, expected {N_PARAMS}")
    return p


def adjacency_masks(q: Query) -> np.ndarray:
    m = np.zeros(q.num_vertices, np.uint32)
    for a, b in np.asarray(q.edges).reshape(-1, 2).tolist():
        if a != b:
            m[a] |= np.uint32(1 << b)
            m[b] |= np.uint32(1 << a)
    return m


def is_connected_order(order, masks) -> bool:
    placed = 0
    for i, u in enumerate(order):
        if i and not (int(masks[u]) & placed):
            return False
        placed |= 1 << int(u)
    return True


def local_moves(order, masks, k: int, rng: np.random.Generator) -> list:
    """Up to k distinct connected orders one move away from `order`: a vertex
    taken from position i and inserted at an earlier position j."""
    n = len(order)
    out, seen = [], {tuple(order)}
    for _ in range(16 * k):
        if len(out) >= k or n < 2:
            break
        i = int(rng.integers(1, n))
        j = int(rng.integers(0, i))
        o = list(order[:j]) + [order[i]] + list(order[j:i]) + list(order[i + 1:])
        t = tuple(o)
        if t not in seen and is_connected_order(o, masks):
            seen.add(t)
            out.append(o)
    return out


def alternative_orders(q: Query, cand, k: int, rng: np.random.Generator, around=None) -> list:
    """Up to k distinct connected orders: half are single moves from `around`
    (the heuristic order) when given; the rest greedy by candidate count
    divided by (1 + alpha * placed neighbours), with multiplicative log-normal
    noise of several strengths, and uniformly random frontier walks."""
    n = q.num_vertices
    masks = [int(x) for x in adjacency_masks(q)]
    cnt = np.maximum(np.asarray(cand, np.float64), 1.0)
    out = local_moves(list(around), masks, k // 2, rng) if around is not None else []
    seen = {tuple(o) for o in out}
    if around is not None:
        seen.add(tuple(around))
    tries = 0
    while len(out) < k and tries < 8 * k:
        tries += 1
        sigma = (0.25, 0.75, 1.5, None)[tries % 4]
        alpha = float(rng.choice([0.0, 0.5, 1.0, 2.0]))
        noisy = rng.random(n) if sigma is None else cnt * np.exp(rng.normal(0, sigma, n))
        placed, order = 0, []
        for i in range(n):
            best, bv = -1, np.inf
            for u in range(n):
                if (placed >> u) & 1 or (i and not (masks[u] & placed)):
                    continue
                back = bin(masks[u] & placed).count("1")
                v = noisy[u] / (1.0 + alpha * back) if sigma is not None else noisy[u]
                if v < bv:
                    best, bv = u, v
            order.append(best)
            placed |= 1 << best
        t = tuple(order)
        if t not in seen:
            seen.add(t)
            out.append(list(order))
    return out


def gsi_completion(prefix, masks, cand) -> list:
    """The order that starts with `prefix` and continues by the heuristic
    order's rule (match/GSI.cu:105-149): the frontier vertex of lowest score,
    a score being the candidate count times 0.9 per placed neighbour (lowest
    id on ties)."""
    n = len(masks)
    score = [float(c) for c in cand]
    placed, order = 0, []

    def place(u):
        nonlocal placed
        order.append(int(u))
        placed |= 1 << int(u)
        for w in range(n):
            if (masks[u] >> w) & 1 and not (placed >> w) & 1:
                score[w] *= 0.9

    for u in prefix:
        place(u)
    while len(order) < n:
        best = -1
        for u in range(n):
            if (placed >> u) & 1 or not (masks[u] & placed):
                continue
            if best < 0 or score[u] < score[best]:
                best = u
        place(best)
    return order


def prefix_orders(q: Query, cand, depth: int = 2) -> list:
    """Every connected order prefix of `depth` vertices, each completed by the
    heuristic rule (gsi_completion): an exhaustive search over the first
    positions, where the choice matters most."""
    masks = [int(x) for x in adjacency_masks(q)]
    n = q.num_vertices
    prefixes = [[u] for u in range(n)]
    for _ in range(min(depth, n) - 1):
        prefixes = [p + [w] for p in prefixes for w in range(n)
                    if w not in p and any((masks[u] >> w) & 1 for u in p)]
    return [gsi_completion(p, masks, cand) for p in prefixes]


@dataclasses.dataclass
class QueryLog:
    query: Query
    candidates: list        # post-filter candidate count per vertex
    count: int
    hash: int
    heuristic_order: list
    heuristic_work: int
    orders: list            # alternatives that finished within the limit
    works: list
    level_counts: list      # per alternative
    aborted: int            # alternatives stopped by the limit

    margin = 0.98  # an alternative replaces the heuristic order below this fraction of its work

    @property
    def best(self):
        """The cheapest order found; the heuristic order unless an alternative
        examined fewer than `margin` times its entries."""
        if self.works and min(self.works) < self.margin * self.heuristic_work:
            i = int(np.argmin(self.works))
            return self.orders[i], self.works[i]
        return self.heuristic_order, self.heuristic_work


def collect_logs(engine: Engine, queries: Sequence[Query], algo: int = ALGO_FUSED, per_query: int = 16,
                 seed: int = 0, batch: int = 2048, heuristic_limit: int = 0, prefix_depth: int = 0) -> list:
    """Order/cost logs for the queries on the engine's resident graph.
    Queries whose heuristic run exceeds heuristic_limit (0: none) are dropped.
    The alternatives are `per_query` sampled orders (alternative_orders), or
    with prefix_depth > 0 every order prefix of that many vertices completed
    by the heuristic rule (prefix_orders).  Alternatives run in batches that
    share one work limit, the largest heuristic work among their queries; an
    alternative costlier than its own query's heuristic is recorded as
    aborted."""
    rng = np.random.default_rng(seed)
    logs = []
    limit = heuristic_limit or UNCAPPED
    for s in range(0, len(queries), batch):
        part = [Query(q.labels, q.edges) for q in queries[s:s + batch]]
        res = engine.match_batch(part, algo=algo, order_source=ORDER_HEURISTIC, max_work=limit)
        alts = []
        for q, r in zip(part, res):
            if r.status != 0:
                continue
            lg = QueryLog(q, list(r.candidates), r.count, r.hash, list(r.order), int(r.work), [], [], [], 0)
            logs.append(lg)
            cands = (prefix_orders(q, r.candidates, prefix_depth) if prefix_depth > 0 else
                     alternative_orders(q, r.candidates, per_query, rng, around=lg.heuristic_order))
            seen = {tuple(lg.heuristic_order)}
            for o in cands:
                if tuple(o) in seen:
                    continue
                seen.add(tuple(o))
                alts.append((Query(q.labels, q.edges, order=np.asarray(o, np.uint32)), lg))
        # sort by the owner's work so each batch's shared limit stays close to its members'
        alts.sort(key=lambda t: t[1].heuristic_work)
        for s2 in range(0, len(alts), batch):
            items = alts[s2:s2 + batch]
            lim = max(max(lg.heuristic_work for _, lg in items), 1)
            rr = engine.match_batch([a for a, _ in items], algo=algo, order_source=ORDER_GIVEN, max_work=lim)
            for (aq, lg), r in zip(items, rr):
                if r.status == ELIMIT or (r.status == 0 and r.work > lg.heuristic_work):
                    lg.aborted += 1
                    continue
                if r.status != 0:
                    raise RuntimeError(f"alternative order failed with status {r.status}")
                if r.count != lg.count or r.hash != lg.hash:
                    raise RuntimeError("an alternative order changed the result")
                lg.orders.append([int(x) for x in aq.order])
                lg.works.append(int(r.work))
                lg.level_counts.append(list(r.level_counts))
    return logs


def cost_targets(lg: QueryLog) -> np.ndarray:
    """Per query vertex u: log2 of (the least work found among the logged
    orders that start with u) / (the heuristic order's work), clipped to
    [-1, 0.5]; 0.5 when no order starting with u finished within the
    heuristic's work.  Lower is a better first vertex, so ordering by the
    lowest predicted value (FSIG_ORDER_LEARNED with learned_prefix) starts
    where the search found the least work."""
    n = lg.query.num_vertices
    best = np.full(n, np.inf)
    h = max(lg.heuristic_work, 1)
    best[lg.heuristic_order[0]] = h
    for o, w in zip(lg.orders, lg.works):
        best[o[0]] = min(best[o[0]], max(w, 1))
    t = np.where(np.isfinite(best), np.log2(np.where(np.isfinite(best), best, 1.0) / h), 0.5)
    return np.clip(t, -1.0, 0.5).astype(np.float32)


def training_set(engine: Engine, logs: Sequence[QueryLog], algo: int = ALGO_FUSED, margin: float | None = None,
                 target: str = "position", oversample: int = 0):
    """(node offsets, features, neighbour masks, targets) for the logs.
    target "position": a vertex's position in the cheapest order found /
    (n - 1), an alternative becoming the target only below margin x the
    heuristic's work; "cost": cost_targets.  With oversample k, a query
    whose cheapest order saves a fraction s of the heuristic's work appears
    1 + round(k * s / 0.2) times."""
    if margin is not None:
        for lg in logs:
            lg.margin = margin
    if oversample:
        rep = []
        for lg in logs:
            saved = 1.0 - min([lg.heuristic_work] + lg.works) / max(lg.heuristic_work, 1)
            rep += [lg] * (1 + int(round(oversample * max(saved, 0.0) / 0.2)))
        logs = rep
    qs = [lg.query for lg in logs]
    feat = engine.mpnn_features(qs, [lg.candidates for lg in logs], algo)
    goff = np.zeros(len(qs) + 1, np.uint32)
    goff[1:] = np.cumsum([q.num_vertices for q in qs])
    nbr = np.concatenate([adjacency_masks(q) for q in qs]) if qs else np.zeros(0, np.uint32)
    tgt = np.zeros(int(goff[-1]), np.float32)
    for i, lg in enumerate(logs):
        if target == "cost":
            tgt[goff[i]:goff[i + 1]] = cost_targets(lg)
            continue
        order, _ = lg.best
        n = len(order)
        for pos, u in enumerate(order):
            tgt[goff[i] + u] = pos / max(n - 1, 1)
    return goff, feat, nbr, tgt


def save_logs(path, logs) -> None:
    """(workload name, QueryLog) pairs as JSON (the data graph's workload,
    query, candidates, heuristic order and work, the finished alternatives
    and their work), to retrain without searching again."""
    import json
    rec = [dict(graph=name, labels=[int(x) for x in lg.query.labels], edges=np.asarray(lg.query.edges).reshape(-1).tolist(),
                candidates=[int(x) for x in lg.candidates], count=int(lg.count), hash=str(int(lg.hash)),
                heuristic_order=[int(x) for x in lg.heuristic_order], heuristic_work=int(lg.heuristic_work),
                orders=lg.orders, works=[int(w) for w in lg.works], aborted=int(lg.aborted)) for name, lg in logs]
    Path(path).write_text(json.dumps(rec))


def load_logs(path) -> list:
    """(workload name, QueryLog) pairs written by save_logs."""
    import json
    out = []
    for r in json.loads(Path(path).read_text()):
        q = Query(np.asarray(r["labels"], np.int32), np.asarray(r["edges"], np.uint32).reshape(-1, 2))
        out.append((r["graph"], QueryLog(q, r["candidates"], r["count"], int(r["hash"]), r["heuristic_order"],
                                         r["heuristic_work"], r["orders"], r["works"], [[] for _ in r["works"]],
                                         r["aborted"])))
    return out


def _subset(goff, feat, nbr, tgt, idx):
    sizes = (goff[1:] - goff[:-1])[idx]
    sel = np.concatenate([np.arange(goff[i], goff[i + 1]) for i in idx]) if len(idx) else np.zeros(0, np.int64)
    off = np.zeros(len(idx) + 1, np.uint32)
    off[1:] = np.cumsum(sizes)
    return off, feat[sel], nbr[sel], tgt[sel]


def train(engine: Engine, data, epochs: int = 60, lr: float = 2e-3, batch_graphs: int = 256, seed: int = 0,
          params: np.ndarray | None = None, verbose: bool = False):
    """Minibatch Adam on the device kernels.  Returns (params, mean loss per epoch)."""
    goff, feat, nbr, tgt = data
    engine.mpnn_set_params(init_params(seed) if params is None else params)
    rng = np.random.default_rng(seed)
    G = len(goff) - 1
    losses = []
    for ep in range(epochs):
        perm = rng.permutation(G)
        tot, nb = 0.0, 0
        for s in range(0, G, batch_graphs):
            loss, _ = engine.mpnn_train_step(*_subset(goff, feat, nbr, tgt, perm[s:s + batch_graphs]), lr=lr)
            tot += loss
            nb += 1
        losses.append(tot / max(nb, 1))
        if verbose:
            print(f"epoch {ep} loss {losses[-1]:.5f}", flush=True)
    return engine.mpnn_get_params(), losses


class LearnedFeed:
    """Serving batches in learned order with the heuristic order as fallback,
    without a batch of its own per fallback: a query over the work limit is
    carried into the next batch with its heuristic order attached (a
    learned-order batch keeps caller-given orders); the ones left after the
    last batch run together at flush().  step(k, batch, results) writes
    (count, hash) pairs into results[k]; a carried query's pair is filled in
    when its later batch returns.  on_stats, when given, receives the engine's
    statistics after every call."""

    def __init__(self, engine: Engine, algo: int = ALGO_FUSED, work_limit: int = 1 << 26, **kw):
        self.engine, self.algo, self.work_limit, self.kw = engine, algo, work_limit, kw
        self.pending = []  # (step, index, query with its heuristic order)

    def _run(self, qs, on_stats):
        rs = self.engine.match_batch(qs, algo=self.algo, order_source=ORDER_LEARNED, max_work=self.work_limit,
                                     **self.kw)
        if on_stats:
            on_stats(self.engine.last_stats())
        return rs

    def _settle(self, rs, results):
        for (k, i, _), r in zip(self.pending, rs):
            if r.status != 0:
                raise RuntimeError(f"fallback query failed with status {r.status}")
            results[k][i] = (r.count, r.hash)
        self.pending = []

    def step(self, k, batch, results, on_stats=None):
        """Runs one batch (plus carried queries); returns (its results, fallbacks)."""
        from . import ALGO_GSI, plan_order
        rs = self._run(list(batch) + [q for _, _, q in self.pending], on_stats)
        self._settle(rs[len(batch):], results)
        rs = rs[: len(batch)]
        results[k] = [(r.count, r.hash) for r in rs]
        for i, r in enumerate(rs):
            if r.status == ELIMIT:
                order = plan_order(batch[i], ALGO_GSI, r.candidates)["order"]
                self.pending.append((k, i, Query(batch[i].labels, batch[i].edges,
                                                 order=np.asarray(order, np.uint32))))
        return rs, sum(1 for r in rs if r.status == ELIMIT)

    def flush(self, results, on_stats=None):
        if self.pending:
            self._settle(self._run([q for _, _, q in self.pending], on_stats), results)


def match_learned(engine: Engine, queries: Sequence[Query], algo: int = ALGO_FUSED, work_limit: int = 0, **kw):
    """Batched learned-order matching with the heuristic order as fallback:
    queries that exceed work_limit under the learned order run again with the
    heuristic order (unlimited).  Returns (results, number of fallbacks)."""
    res = engine.match_batch(queries, algo=algo, order_source=ORDER_LEARNED, max_work=work_limit, **kw)
    redo = [i for i, r in enumerate(res) if r.status == ELIMIT]
    if redo:
        again = engine.match_batch([queries[i] for i in redo], algo=algo, order_source=ORDER_HEURISTIC, **kw)
        for i, r in zip(redo, again):
            res[i] = r
    return res, len(redo)


# ---------------------------------------------------------------------------
# training the packaged network: logs on the mid-scale graphs
# ---------------------------------------------------------------------------
def training_workloads():
    """(name, graph builder, query specs, work limit, queries kept) of the logs
    the packaged network is trained on: the two graphs of the benchmarked
    serving workloads with queries of their shapes drawn from seeds apart from
    the benchmark's (workloads.candidate_specs of ranks 40 and 41; the
    benchmark's manifests use rank 0): the 2^22-vertex Chung-Lu graph with
    12-32-vertex dense walks on labels >= 8, and the 320k-vertex Chung-Lu graph
    with 4-32-vertex dense and sparse walks on labels >= 4.  Only queries whose
    heuristic run stays within the benchmark's selection budget are kept.  The
    unlabeled 2^20-vertex R-MAT graph is not logged: its 5-vertex patterns
    have about 1e15 embeddings each."""
    from . import workloads as W
    c5 = W.candidate_specs("c5", rank=40)[0][0]
    dense, sparse = W.candidate_specs("c4", rank=41)[0]
    c4 = [x for pair in zip(dense[:4096], sparse[:4096]) for x in pair]
    return [("c5", lambda: W.build_graph("c5"), c5, W.WORK_BUDGET, 2048),
            ("c4", lambda: W.build_graph("c4"), c4, W.WORK_BUDGET, 512)]


def main(argv=None):
    import argparse
    import time

    from . import gen_queries, select_within_budget
    ap = argparse.ArgumentParser(description="Train the order-scoring network on the engine's own logs.")
    ap.add_argument("--out", default=str(WEIGHTS))
    ap.add_argument("--prefix-depth", type=int, default=2,
                    help="alternatives: every order prefix of this many vertices completed by the heuristic rule "
                         "(0: --per-query sampled orders instead)")
    ap.add_argument("--per-query", type=int, default=16)
    ap.add_argument("--queries", type=int, default=0, help="queries logged per workload (default: per workload)")
    ap.add_argument("--target", default="position", choices=["cost", "position"],
                    help="cost: log work ratio of the best order starting at each vertex; position: its position "
                         "in the cheapest order found")
    ap.add_argument("--oversample", type=int, default=4,
                    help="repeat queries by the share of work their best order saves (0: no repeats)")
    ap.add_argument("--save-logs", default="", help="write the logs here (JSON)")
    ap.add_argument("--logs", default="", help="train on these saved logs instead of logging again")
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--work-limit", type=int, default=0,
                    help="drop queries whose heuristic run examines more (default: per workload)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--margin", type=float, default=0.98,
                    help="an alternative order becomes the target below this fraction of the heuristic's work")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    logs = []
    all_logs = []
    with Engine(args.device, arena_bytes=48 << 30) as e:
        t0 = time.time()
        if args.logs:
            from . import workloads as W
            # features come from the engine's candidate counts: each log's graph must be resident
            by_graph = {}
            for name, x in load_logs(args.logs):
                by_graph.setdefault(name, []).append(x)
            for name, part in by_graph.items():
                e.load_graph(W.build_graph(name))
                logs.append((part, training_set(e, part, margin=args.margin, target=args.target,
                                                oversample=args.oversample)))
        for name, build, specs, limit, keep in ([] if args.logs else training_workloads()):
            g = build()
            csr = g.csr()
            e.load_graph(g)
            want = args.queries or keep
            qs = []
            for i in range(0, len(specs), 2048):
                qs += select_within_budget(e, gen_queries(g, specs[i:i + 2048], csr=csr), want - len(qs),
                                           args.work_limit or limit)
                if len(qs) >= want:
                    break
            print(f"[learn] {name}: {len(qs)} queries within the work limit, {time.time() - t0:.1f}s", flush=True)
            lg = collect_logs(e, qs, per_query=args.per_query, seed=args.seed, prefix_depth=args.prefix_depth,
                              batch=1024)
            gain = sum(x.heuristic_work for x in lg) / max(sum(x.best[1] for x in lg), 1)
            print(f"[learn] {name}: {len(lg)} queries logged, best/heuristic total work 1/{gain:.3f}, "
                  f"{time.time() - t0:.1f}s", flush=True)
            all_logs += [(name, x) for x in lg]
            logs.append((lg, training_set(e, lg, margin=args.margin, target=args.target,
                                          oversample=args.oversample)))
        if args.save_logs and all_logs:
            save_logs(args.save_logs, all_logs)
        goff = np.zeros(1, np.uint32)
        feats, nbrs, tgts = [], [], []
        for _, (o, f, nb, t) in logs:
            goff = np.concatenate([goff, goff[-1] + o[1:]])
            feats.append(f)
            nbrs.append(nb)
            tgts.append(t)
        data = (goff, np.concatenate(feats), np.concatenate(nbrs), np.concatenate(tgts))
        params, losses = train(e, data, epochs=args.epochs, lr=args.lr, seed=args.seed)
        print(f"[learn] trained {len(goff) - 1} graphs, loss {losses[0]:.4f} -> {losses[-1]:.4f}, "
              f"{time.time() - t0:.1f}s", flush=True)
        np.save(args.out, params)
        print(f"[learn] wrote {args.out}", flush=True)


if __name__ == "__main__":
    main()
