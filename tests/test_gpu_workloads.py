"""Parity on the benchmarked workloads at full size, against the oracle.

The queries come from the workload manifests (rebuilt by the generators, the
graphs' digests checked first); the oracle's counts and set hashes for them
were recorded by tests/golden/make_workload_golden.py: every query with at
most 2e7 embeddings of

  config 2  (320k-vertex Chung-Lu graph, 200 queries of 8 vertices)
  config 4  (the same graph, 4,096 queries of 4-32 vertices)
  config 5  (2^22-vertex Chung-Lu graph, 2,048 queries of 12-32 vertices)

They run through the batched path as the benchmark runs them (batches of up
to 512 queries, one CUDA graph each) and, for config 5, with ordinary
launches too; config 2's also through the single-query path of both
reference algorithms.  Semantics: injective, label-preserving, non-induced
(match/MMatch_kernels.cuh:641-654, match/GSI_kernels.cuh:199-213).
"""
import json

import pytest

import fsig_gb300 as F
from conftest import GOLDEN
from fsig_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def records():
    return json.loads((GOLDEN / "workload_oracle.json").read_text())


def _sample(records, name):
    w = W.load(name)
    assert w.manifest["graph_digest"] == records["graphs"][name]
    r = records["workloads"][name]
    qs = [w.batches[b][i] for b, i in zip(r["batch"], r["index"])]
    want = [(c, int(h)) for c, h in zip(r["count"], r["hash"])]
    return w, qs, want


@pytest.mark.parametrize("name,min_queries", [("c2", 100), ("c4", 3000), ("c5", 1500)])
def test_workload_matches_oracle(engine, records, name, min_queries):
    w, qs, want = _sample(records, name)
    assert len(qs) >= min_queries
    engine.load_graph(w.graph)
    modes = (True, False) if name == "c5" else (True,)
    for use_graph in modes:
        got = []
        for k in range(0, len(qs), 512):
            rs = engine.match_batch(qs[k:k + 512], algo=F.ALGO_FUSED, use_graph=use_graph)
            assert [r.status for r in rs] == [0] * len(rs)
            got += [(r.count, r.hash) for r in rs]
        bad = [i for i, (a, b) in enumerate(zip(got, want)) if a != b]
        assert not bad, f"{len(bad)} of {len(qs)} differ, first {bad[:5]}"
    if name == "c2":
        for q, (c, h) in zip(qs[:40], want[:40]):
            for algo in (F.ALGO_FSIG, F.ALGO_GSI):
                r = engine.match(q, algo)
                assert (r.count, r.hash) == (c, h)
