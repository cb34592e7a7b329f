"""Parity on the benchmarked workloads at full size, against the oracle.

The queries come from the workload manifests (rebuilt by the generators, the
graphs' digests checked first); the oracle's counts and set hashes for them
were recorded by tests/golden/make_workload_golden.py:

  config 2  (320k-vertex Chung-Lu graph, 8-vertex queries): every manifest
            query with at most 2e7 embeddings
  config 4  (the same graph, 4-32-vertex queries): a 16-query sample
  config 5  (2^22-vertex Chung-Lu graph, 12-32-vertex queries): 4 queries

Each sample runs through the batched path (as one CUDA graph, and with
ordinary launches) and, for config 2, through the single-query path of both
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
    recs = [r for r in records["queries"] if r["workload"] == name]
    qs = [w.batches[r["batch"]][r["index"]] for r in recs]
    want = [(r["count"], int(r["hash"])) for r in recs]
    return w, qs, want


@pytest.mark.parametrize("name,min_queries", [("c2", 100), ("c4", 16), ("c5", 4)])
def test_workload_sample_matches_oracle(engine, records, name, min_queries):
    w, qs, want = _sample(records, name)
    assert len(qs) >= min_queries
    engine.load_graph(w.graph)
    for use_graph in (True, False):
        rs = engine.match_batch(qs, algo=F.ALGO_FUSED, use_graph=use_graph)
        assert [r.status for r in rs] == [0] * len(qs)
        assert [(r.count, r.hash) for r in rs] == want
    if name == "c2":
        for q, (c, h) in zip(qs[:40], want[:40]):
            for algo in (F.ALGO_FSIG, F.ALGO_GSI):
                r = engine.match(q, algo)
                assert (r.count, r.hash) == (c, h)
