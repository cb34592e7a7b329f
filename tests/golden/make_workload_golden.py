"""Oracle results for the benchmarked workloads at full size.

The GPU tests (tests/test_gpu_workloads.py) compare the engine with these
records instead of running the CPU matcher on the GPU machine.  For each of the
config-2, config-4 and config-5 manifests (320k-vertex Chung-Lu graph with
200 8-vertex and 4,096 4-32-vertex queries; 2^22-vertex Chung-Lu graph with
2,048 12-32-vertex queries) it holds every query whose embedding count (as the
manifest records it) is at most 2e7: its batch and index in the batch, and
the oracle's count and set hash.  The file also records each graph's digest,
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

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from fsig_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

LIMIT = 20_000_000
OUT = HERE / "workload_oracle.json"


def pick(w: W.Workload) -> list:
    return [(b, i) for b in range(len(w.batches)) for i, c in enumerate(w.counts[b]) if c <= LIMIT]


def main() -> None:
    out = {"limit": LIMIT, "graphs": {}, "workloads": {}}
    threads = os.cpu_count() or 1
    for name in ("c2", "c4", "c5"):
        t = time.time()
        w = W.load(name)
        out["graphs"][name] = w.manifest["graph_digest"]
        off, adj = w.csr
        rec = {"batch": [], "index": [], "count": [], "hash": []}
        for b, i in pick(w):
            q = w.batches[b][i]
            c, h, _ = O.match(w.graph.labels, off, adj, q.labels, q.edges, threads=threads)
            rec["batch"].append(b)
            rec["index"].append(i)
            rec["count"].append(int(c))
            rec["hash"].append(str(int(h)))
        out["workloads"][name] = rec
        print(f"{name}: {len(rec['count'])} queries, {time.time() - t:.0f}s", flush=True)
    OUT.write_text(json.dumps(out, separators=(",", ":")))


if __name__ == "__main__":
    main()
