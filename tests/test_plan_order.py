"""Join orders, query decomposition and equivalence classes against the
reference's own host code (GSI::generate_join_order, MMatch::
decompose_query_graph / find_equivalent_classes / generate_join_order), for
seeded candidate counts including all-tied and many-tied cases."""
import pytest

import fsig_gb300 as F
from conftest import GOLDEN


def cases(golden):
    for name, rec in sorted(golden["queries"].items()):
        for i, c in enumerate(rec["cases"]):
            yield name, rec["file"], i, c


def test_orders_match_reference(golden):
    n = 0
    for name, f, i, c in cases(golden):
        q = F.read_query(GOLDEN / f)
        g = F.plan_order(q, F.ALGO_GSI, c["counts"])
        m = F.plan_order(q, F.ALGO_FSIG, c["counts"])
        assert g["order"] == c["gsi_order"], (name, i)
        assert m["order"] == c["mm_order"], (name, i)
        assert m["types"] == c["mm_types"], (name, i)
        assert m["classes"] == c["mm_classes"], (name, i)
        n += 1
    assert n >= 50


def test_orders_are_connected(golden):
    for name, f, i, c in cases(golden):
        q = F.read_query(GOLDEN / f)
        adj = {u: set() for u in range(q.num_vertices)}
        for a, b in q.edges.tolist():
            adj[a].add(b)
            adj[b].add(a)
        for algo in (F.ALGO_GSI, F.ALGO_FSIG):
            o = F.plan_order(q, algo, c["counts"])["order"]
            assert sorted(o) == list(range(q.num_vertices))
            for k in range(1, len(o)):
                assert adj[o[k]] & set(o[:k]), (name, algo, o)


def test_rejects_disconnected_query():
    import numpy as np
    q = F.Query(np.array([0, 0, 0, 0], np.int32), np.array([[0, 1], [2, 3]], np.uint32))
    with pytest.raises(F.FsigError):
        F.plan_order(q, F.ALGO_GSI, [1, 1, 1, 1])
