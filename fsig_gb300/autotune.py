"""Autotuner of the batched path's launch knobs, by measurement.

The enumeration kernel's behaviour on a workload depends on five knobs of
``fsig_batch_opts``:

* ``warps_per_block`` - block size of the persistent enumeration launch
  (warps that share an SM's blocks);
* ``chunk`` - tasks a warp takes per grab of the shared task counter;
* ``split_len`` - driver entries per task range (the unit of root tasks and
  hand-offs, and so of load balance);
* ``split_cycles`` - SM cycles a task runs before its unexplored frontier may
  be handed to idle warps;
* ``isect`` - the set-intersection strategy of the membership tests: 0
  every lane binary-searches the segment alone, 1 warp-cooperative 32-ary
  window search (galloping-like), 2 adaptive (the 32 entries after a
  segment's cursor first, merge-like, then the window search), 3 the tile
  search for segments whose rest fits 32 entries and per-lane binary search
  for longer ones.

When the batch refines candidates (``refine_iters`` > 0) one more joins:

* ``refine_coop`` - warps per candidate in the refinement: a candidate whose
  neighbour segment is longer than this is scanned by the whole warp
  (coalesced, one ballot per 32 entries), shorter ones by the candidate's own
  lane.

With ``order_source = ORDER_LEARNED`` two more knobs join the grid:

* ``learned_window`` - positions a vertex may move away from the heuristic
  order;
* ``learned_prefix`` - positions the network chooses before the heuristic
  rule takes over.

Both change the orders and with them the work; a query whose learned order
goes over ``max_work`` is run again in heuristic order (as serving does), and
that run's device time counts towards the trial.

``tune`` runs coordinate descent over a small grid on a sample batch: one knob
at a time, each value timed by device time (CUDA events of the engine) as the
median of ``repeats`` runs, keeping the best before moving to the next knob.
Every trial's counts and hashes must equal the first run's; a knob choice
never changes results, so a mismatch is an engine fault and raises.
"""
from __future__ import annotations

import statistics
from typing import Sequence

from . import ALGO_FUSED, ELIMIT, ORDER_HEURISTIC, ORDER_LEARNED, Engine, Query

GRID = {
    "warps_per_block": [4, 8],
    "chunk": [1, 2, 4, 8],
    "split_len": [64, 128, 256, 512, 1024],
    "split_cycles": [1000, 4000, 16000, 64000],
    "isect": [0, 1, 2, 3],
}
DEFAULTS = {"warps_per_block": 8, "chunk": 1, "split_len": 256, "split_cycles": 4000, "isect": 0}
REFINE_GRID = {"refine_coop": [8, 32, 128, 0xFFFFFFFF]}
REFINE_DEFAULTS = {"refine_coop": 32}
LEARNED_GRID = {"learned_window": [1, 2, 4, 32], "learned_prefix": [1, 2, 32]}
LEARNED_DEFAULTS = {"learned_window": 32, "learned_prefix": 32}


def _device_ms(engine: Engine) -> float:
    st = engine.last_stats()
    return st["ms_filter"] + st["ms_join"]


def _time(engine: Engine, batch, kw, repeats: int, want):
    ts = []
    for _ in range(repeats):
        rs = engine.match_batch(batch, **kw)
        ms = _device_ms(engine)
        got = [(r.count, r.hash) for r in rs]
        over = [i for i, r in enumerate(rs) if r.status == ELIMIT]
        if over and kw.get("order_source") == ORDER_LEARNED:
            # serving runs these again in heuristic order
            again = engine.match_batch([batch[i] for i in over], **dict(kw, order_source=ORDER_HEURISTIC))
            ms += _device_ms(engine)
            for i, r in zip(over, again):
                got[i] = (r.count, r.hash)
        if want is not None and got != want:
            raise RuntimeError(f"launch knobs {kw} changed the results")
        ts.append(ms)
    return statistics.median(ts), got


def tune(engine: Engine, batch: Sequence[Query], algo: int = ALGO_FUSED, order_source: int = ORDER_HEURISTIC,
         repeats: int = 2, rounds: int = 1, **fixed):
    """Best knobs for the batch: (dict of knobs, list of (knobs, ms) trials).
    `fixed` (e.g. max_work, use_graph) is passed to every run unchanged."""
    base = dict(algo=algo, order_source=order_source, **fixed)
    learned = order_source == ORDER_LEARNED
    refines = fixed.get("refine_iters", -1) > 0 or (algo == 1 and fixed.get("refine_iters", -1) != 0)
    grid = {**GRID, **(LEARNED_GRID if learned else {}), **(REFINE_GRID if refines else {})}
    best = {**DEFAULTS, **(LEARNED_DEFAULTS if learned else {}), **(REFINE_DEFAULTS if refines else {})}
    engine.match_batch(batch, **base, **best)  # warm-up
    best_ms, want = _time(engine, batch, {**base, **best}, repeats, None)
    trials = [(dict(best), best_ms)]
    for _ in range(rounds):
        for knob, values in grid.items():
            for v in values:
                if v == best[knob]:
                    continue
                cand = dict(best, **{knob: v})
                ms, _ = _time(engine, batch, {**base, **cand}, repeats, want)
                trials.append((cand, ms))
                if ms < best_ms:
                    best, best_ms = cand, ms
    return best, trials
