"""Oracle results for samples of the benchmarked workloads at full size.

The GPU tests (tests/test_gpu_workloads.py) compare the engine with these
records instead of running the CPU matcher on the GPU machine:

  c2  every query of the config-2 manifest (320k-vertex Chung-Lu graph, 200
      queries of 8 vertices) whose embedding count is at most 2e7
  c4  16 queries of the config-4 manifest, a seeded sample among those with
      at most 2e7 embeddings
  c5  the first 4 queries of batch 0's reference subset of the config-5
      manifest (2^22-vertex graph, 12-32-vertex queries)

Each record holds the workload, the batch and the query's index in it, and
the oracle's count and set hash; the file also records each graph's digest,
which the tests check first.  The queries and graphs are rebuilt from the
manifests by the generators (identical on x86-64 and AArch64).

    python tests/golden/make_workload_golden.py
"""
from __future__ import annotations

import json
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from fsig_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

LIMIT = 20_000_000
OUT = HERE / "workload_oracle.json"


def pick(name: str, w: W.Workload) -> list:
    if name == "c2":
        return [(b, i) for b in range(len(w.batches)) for i, c in enumerate(w.counts[b]) if c <= LIMIT]
    if name == "c4":
        pool = [(b, i) for b in range(len(w.batches)) for i, c in enumerate(w.counts[b]) if c <= LIMIT]
        rng = np.random.default_rng(404)
        return sorted(pool[j] for j in rng.choice(len(pool), 16, replace=False))
    if name == "c5":
        return [(0, i) for i in w.ref_subset[0][:4]]
    raise ValueError(name)


def main() -> None:
    out = {"limit": LIMIT, "graphs": {}, "queries": []}
    threads = os.cpu_count() or 1
    for name in ("c2", "c4", "c5"):
        t = time.time()
        w = W.load(name)
        out["graphs"][name] = w.manifest["graph_digest"]
        off, adj = w.csr
        for b, i in pick(name, w):
            q = w.batches[b][i]
            c, h, _ = O.match(w.graph.labels, off, adj, q.labels, q.edges, threads=threads)
            out["queries"].append({"workload": name, "batch": b, "index": i, "count": int(c), "hash": str(int(h))})
        print(f"{name}: {sum(1 for r in out['queries'] if r['workload'] == name)} queries, "
              f"{time.time() - t:.0f}s", flush=True)
    OUT.write_text(json.dumps(out, indent=0))


if __name__ == "__main__":
    main()
