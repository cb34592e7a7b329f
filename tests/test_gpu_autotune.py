"""Autotuner of the launch knobs: every knob setting it tries returns the
same counts and hashes, and it returns a setting from its grid."""
import pytest

import fsig_gb300 as F
from fsig_gb300 import autotune

pytestmark = pytest.mark.gpu


def test_autotune_on_a_small_batch(engine):
    lab = F.gen_labels(20000, 8, "zipf", seed=4)
    g = F.gen_chung_lu(20000, 80000, 2.1, seed=4, labels=lab)
    off, adj = g.csr()
    engine.load_graph(g)
    qs = [F.gen_query(g, 6 + i % 6, F.QUERY_DENSE if i % 2 else F.QUERY_SPARSE, seed=300 + i, csr=(off, adj))
          for i in range(48)]
    qs = F.select_within_budget(engine, qs, 32, 1 << 22)
    base = [(r.count, r.hash) for r in engine.match_batch(qs)]
    best, trials = autotune.tune(engine, qs, repeats=1, use_graph=True)
    assert set(best) == set(autotune.GRID)
    assert all(best[k] in autotune.GRID[k] for k in best)
    # every grid value is tried once per knob (the starting value again when
    # an earlier value of the same knob displaced it)
    assert 1 + sum(len(v) - 1 for v in autotune.GRID.values()) <= len(trials) <= 1 + sum(map(len, autotune.GRID.values()))
    assert [(r.count, r.hash) for r in engine.match_batch(qs, **best)] == base
    for wpb in (1, 2, 4):
        assert [(r.count, r.hash) for r in engine.match_batch(qs, warps_per_block=wpb)] == base
