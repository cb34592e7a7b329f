"""The benchmark workloads on the CPU: the generators reproduce every
manifest's graph bit for bit (the manifests were written on the Arm GPU machine,
these tests also run on x86-64), and the manifests are well formed.  The
config-3 graph has no manifest; its digest is pinned here."""
import json

import numpy as np
import pytest

from fsig_gb300 import workloads as W

# sha256 of labels + edges of the R-MAT 2^20 / 2^24 graph (seed 3), the same
# on x86-64 and AArch64
C3_DIGEST = "3dae76bb60e5337ee211f874c3e59e32c9d808bc8975131fb1cfb8e538a8d1a2"
WITH_MANIFEST = ["c1", "c2", "c4", "c5"]


@pytest.mark.parametrize("name", WITH_MANIFEST)
def test_generator_reproduces_manifest_graph(name):
    m = json.loads(W.manifest_path(name).read_text())
    assert W.graph_digest(W.build_graph(name)) == m["graph_digest"]


def test_config3_graph_digest():
    g = W.build_graph("c3")
    assert g.num_vertices == 1 << 20 and g.num_edges == 1 << 24
    e = g.edges
    assert (e[:, 0] < e[:, 1]).all()  # canonical, no self-loops
    assert (g.labels == 0).all()
    assert W.graph_digest(g) == C3_DIGEST


@pytest.mark.parametrize("name", WITH_MANIFEST)
def test_manifest_shape(name):
    m = json.loads(W.manifest_path(name).read_text())
    pools, wants, bsize = W.candidate_specs(name)
    total = sum(wants)
    batches = m["batches"]
    assert sum(len(b["specs"]) for b in batches) == total
    assert all(len(b["specs"]) == bsize for b in batches[:-1])
    for b in batches:
        n = len(b["specs"])
        assert len(b["work"]) == len(b["counts"]) == len(b["hashes"]) == n
        assert max(b["work"]) <= m["work_budget"] == W.WORK_BUDGET
        assert b["ref_subset"] and sorted(set(b["ref_subset"])) == b["ref_subset"]
        assert 0 <= b["ref_subset"][0] and b["ref_subset"][-1] < n
    assert len(m["tune_specs"]) == bsize
    # the specs are drawn, in order, from the workload's candidate pools
    pool_specs = {tuple(s) for p in pools for s in p}
    timed = [tuple(s) for b in batches for s in b["specs"]]
    tune = [tuple(s) for s in m["tune_specs"]]
    assert set(timed) <= pool_specs and set(tune) <= pool_specs
    assert not set(timed) & set(tune)


def test_load_rebuilds_queries():
    w = W.load("c1")
    assert len(w.batches) == 1 and len(w.batches[0]) == 100
    assert all(q.num_vertices == 4 for q in w.batches[0])
    # every query embeds at the data vertices it was drawn from
    off, adj = w.csr
    for q in w.batches[0][:20]:
        assert (w.graph.labels[q.source] == q.labels).all()
        for a, b in np.asarray(q.edges).tolist():
            x, y = q.source[a], q.source[b]
            assert y in adj[off[x]:off[x + 1]]


def test_rank_order():
    assert W.rank_order(4, 0) == [0, 1, 2, 3]
    assert W.rank_order(4, 5) == [1, 2, 3, 0]
    assert W.rank_order(1, 3) == [0]
