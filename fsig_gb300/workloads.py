"""The benchmark workloads: seeded synthetic data graphs and query sets with
the shapes of the five configurations, and the manifests that fix which
queries each workload runs.

No dataset is available, so seeded generators (libfsig_gen.so, host code that
gives bit-identical graphs on x86-64 and AArch64) stand in:

  c1  R-MAT 10,000 / 50,000 (a .57, b .19, c .19), seed 1, 8 uniform labels;
      100 induced random-walk queries of 4 vertices
  c2  Chung-Lu 320,000 / 1,050,000, exponent 2.1, seed 2, 16 Zipf(1.0)
      labels; 200 queries of 8 vertices, 100 dense and 100 sparse walks
  c3  R-MAT 2^20 / 2^24 distinct edges, seed 3, no self-loops, unlabeled;
      the five 5-vertex patterns (K4 plus a pendant vertex, the 5-cycle, the
      house, two seeded random connected graphs)
  c4  the c2 graph; 4,096 queries of 4-32 vertices, half dense, half sparse,
      batches of 512
  c5  Chung-Lu 2^22 / 2^26, exponent 2.0, seed 5, 32 Zipf labels; 2,048
      dense queries of 12-32 vertices, batches of 512

Random-walk queries of these sizes over all labels of the large graphs have
more than 10^9 partial embeddings each, beyond any exact matcher; a workload
therefore keeps, in a seeded order of candidates, the first ones whose
enumeration under the heuristic order examines at most WORK_BUDGET driver
entries (a property of query and graph alone).  Making that choice needs the
GPU engine; it is made once and written to a manifest
(fsig_gb300/manifests/<name>.json) that lists, in batch order, each query's
generator spec (vertices, walk mode, seed, label floor) with the work and
embedding count and set hash measured then, and for every batch the fixed
subset of its queries that the CPU reference arm times (the first queries in
batch order until their work adds up to REF_WORK).  ``load(name)`` rebuilds
the graph and the queries from the manifest with the host generators alone,
and checks the graph's digest, so both benchmark arms and the tests run the
same queries without opening the engine.

    python -m fsig_gb300.workloads --write c5 c4 c2 c1 --out DIR   (on a GPU machine)
"""
from __future__ import annotations

import argparse
import hashlib
import json
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import (ALGO_FUSED, QUERY_DENSE, QUERY_INDUCED, QUERY_SPARSE, Graph, Query, gen_chung_lu, gen_labels,
               gen_queries, gen_rmat)

MANIFESTS = Path(__file__).resolve().parent / "manifests"
WORK_BUDGET = 1 << 26
NAMES = ("c1", "c2", "c3", "c4", "c5")

GRAPH_DESC = {
    "c1": "R-MAT 10k V / 50k E, 8 uniform labels",
    "c2": "Chung-Lu 320k V / 1.05M E, exp 2.1, 16 Zipf labels",
    "c3": "R-MAT 2^20 V / 2^24 E, seed 3, unlabeled",
    "c4": "Chung-Lu 320k V / 1.05M E, exp 2.1, 16 Zipf labels",
    "c5": "Chung-Lu 2^22 V / 2^26 E, exp 2.0, 32 Zipf labels",
}


def build_graph(name: str) -> Graph:
    """The workload's data graph (deterministic, platform-independent)."""
    if name == "c5":
        lab = gen_labels(1 << 22, 32, "zipf", seed=5)
        return gen_chung_lu(1 << 22, 1 << 26, 2.0, seed=5, labels=lab)
    if name in ("c4", "c2"):
        lab = gen_labels(320000, 16, "zipf", seed=2)
        return gen_chung_lu(320000, 1050000, 2.1, seed=2, labels=lab)
    if name == "c3":
        return gen_rmat(1 << 20, 1 << 24, 0.57, 0.19, 0.19, seed=3)
    if name == "c1":
        lab = gen_labels(10000, 8, "uniform", seed=1)
        return gen_rmat(10000, 50000, 0.57, 0.19, 0.19, seed=1, labels=lab)
    raise ValueError(f"unknown workload {name}")


def graph_digest(g: Graph) -> str:
    """sha256 of the labels (int32) and the edge list (uint32 pairs)."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(g.labels, np.int32).tobytes())
    h.update(np.ascontiguousarray(g.edges, np.uint32).tobytes())
    return h.hexdigest()


# ---------------------------------------------------------------------------
# config 3: the unlabeled 5-vertex patterns
# ---------------------------------------------------------------------------
def random_connected(seed: int) -> list:
    """A seeded random connected graph on 5 vertices (each pair an edge with
    probability 1/2, redrawn until connected)."""
    rng = np.random.default_rng(seed)
    while True:
        e = {(i, j) for i in range(5) for j in range(i + 1, 5) if rng.random() < 0.5}
        adj = {i: set() for i in range(5)}
        for a, b in e:
            adj[a].add(b)
            adj[b].add(a)
        seen, todo = {0}, [0]
        while todo:
            for w in adj[todo.pop()]:
                if w not in seen:
                    seen.add(w)
                    todo.append(w)
        if len(seen) == 5:
            return sorted(e)


PATTERNS = {
    "k4_pendant": [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3), (0, 4)],
    "c5": [(0, 1), (1, 2), (2, 3), (3, 4), (4, 0)],
    "house": [(0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (1, 4)],
    "random_a": random_connected(31),
    "random_b": random_connected(32),
}


def pattern(name_or_edges, n: int = 5) -> Query:
    edges = PATTERNS[name_or_edges] if isinstance(name_or_edges, str) else name_or_edges
    return Query(np.zeros(n, np.int32), np.asarray(edges, np.uint32).reshape(-1, 2))


# ---------------------------------------------------------------------------
# query candidates and manifests
# ---------------------------------------------------------------------------
def candidate_specs(name: str, rank: int = 0):
    """(pools of generator specs in a seeded order, queries wanted per pool,
    batch size).  A spec is (vertices, walk mode, seed[, label floor])."""
    rng = np.random.default_rng(1000 + rank)
    base = 1_000_000 * (rank + 1)
    if name == "c5":
        sizes = rng.integers(12, 33, 32768)
        return [[(int(n), QUERY_DENSE, base + i, 8) for i, n in enumerate(sizes)]], [2048], 512
    if name == "c4":
        sizes = rng.integers(4, 33, 32768)
        dense = [(int(n), QUERY_DENSE, base + i, 4) for i, n in enumerate(sizes)]
        sparse = [(int(n), QUERY_SPARSE, base + 500_000 + i, 4) for i, n in enumerate(sizes)]
        return [dense, sparse], [2048, 2048], 512
    if name == "c2":
        dense = [(8, QUERY_DENSE, base + i, 4) for i in range(32768)]
        sparse = [(8, QUERY_SPARSE, base + 500_000 + i, 4) for i in range(32768)]
        return [dense, sparse], [100, 100], 200
    if name == "c1":
        return [[(4, QUERY_INDUCED, base + i) for i in range(1000)]], [100], 100
    raise ValueError(f"workload {name} has no query candidates")


@dataclass
class Workload:
    name: str
    graph: Graph
    csr: tuple
    desc: str
    batches: list                      # lists of Query, in batch order
    specs: list                        # per batch, the generator specs
    work: list                         # per batch, heuristic-order work of each query (at manifest time)
    counts: list                       # per batch, embedding count of each query (at manifest time)
    hashes: list                       # per batch, set hash of each query (at manifest time)
    ref_subset: list                   # per batch, indices of the queries the CPU arm times
    tune: list                         # a further batch of selected queries that is never timed
    manifest: dict = field(default_factory=dict)


def manifest_path(name: str, manifest_dir=None) -> Path:
    return Path(manifest_dir or MANIFESTS) / f"{name}.json"


def rank_order(n_batches: int, rank: int) -> list:
    """Batch order of replica `rank`: the manifest's batches starting at batch
    rank (mod their number), so that replicas work on different queries."""
    k = rank % max(n_batches, 1)
    return [(k + i) % n_batches for i in range(n_batches)]


def load(name: str, rank: int = 0, check_digest: bool = True, manifest_dir=None) -> Workload:
    """Graph and query batches of a workload, rebuilt from its manifest with
    the host generators (no GPU).  Rank r > 0 (replicas under torchrun) runs
    the same batches starting at batch r."""
    m = json.loads(manifest_path(name, manifest_dir).read_text())
    g = build_graph(name)
    if check_digest:
        d = graph_digest(g)
        if d != m["graph_digest"]:
            raise RuntimeError(f"workload {name}: generated graph digest {d[:16]} differs from the manifest's "
                               f"{m['graph_digest'][:16]}: the generators are not reproducing the graph")
    csr = g.csr()
    batches, specs, work, counts, hashes, subset = [], [], [], [], [], []
    for b in m["batches"]:
        sp = [tuple(s) for s in b["specs"]]
        batches.append(gen_queries(g, sp, csr=csr))
        specs.append(sp)
        work.append(list(b["work"]))
        counts.append(list(b["counts"]))
        hashes.append([int(h) for h in b["hashes"]])
        subset.append(list(b["ref_subset"]))
    tune = gen_queries(g, [tuple(s) for s in m["tune_specs"]], csr=csr) if m.get("tune_specs") else []
    if rank and len(batches) > 1:
        order = rank_order(len(batches), rank)
        batches, specs, work, counts, hashes, subset = ([x[i] for i in order] for x in
                                                        (batches, specs, work, counts, hashes, subset))
    return Workload(name, g, csr, GRAPH_DESC[name], batches, specs, work, counts, hashes, subset, tune, m)


def _select(engine, g, csr, pools, wants):
    """For each pool, the first `want` specs whose heuristic-order enumeration
    examines at most WORK_BUDGET driver entries, with that work and count."""
    picked_all = []
    for pool, want in zip(pools, wants):
        picked = []
        for i in range(0, len(pool), 2048):
            part = pool[i:i + 2048]
            cand = gen_queries(g, part, csr=csr)
            for j in range(0, len(cand), 512):
                rs = engine.match_batch(cand[j:j + 512], algo=ALGO_FUSED, max_work=WORK_BUDGET)
                for s, r in zip(part[j:j + 512], rs):
                    if r.status == 0 and len(picked) < want:
                        picked.append((s, int(r.work), int(r.count)))
            if len(picked) >= want:
                break
        if len(picked) < want:
            raise RuntimeError(f"only {len(picked)} of {want} candidates fit the work budget")
        picked_all.append(picked)
    return picked_all


def _ref_subset(work, target_work: int, per_query_work: int):
    """The batch's queries the CPU reference arm times: in batch order, those
    whose heuristic work is at most per_query_work, until their work adds up
    to target_work (the CPU matcher's time follows the work closely)."""
    idx, tot = [], 0
    for i, w in enumerate(work):
        if w > per_query_work:
            continue
        idx.append(i)
        tot += w
        if tot >= target_work:
            break
    return idx


REF_WORK = 1 << 26          # per batch: the CPU arm's sample adds up to about this much work
REF_QUERY_WORK = 1 << 26    # ... from queries of at most this much work each (all of a workload's)


def make_manifest(engine, name: str, ref_work: int = REF_WORK, ref_query_work: int = REF_QUERY_WORK) -> dict:
    t = time.time()
    g = build_graph(name)
    csr = g.csr()
    engine.load_graph(g)
    pools, wants, bsize = candidate_specs(name)
    # one more batch's worth of queries, for tuning launch knobs off the timed batches
    extra = [w + bsize // len(wants) for w in wants]
    picked = _select(engine, g, csr, pools, extra)
    tune = [x for p, w in zip(picked, wants) for x in p[w:]]
    picked = [p[:w] for p, w in zip(picked, wants)]
    mixed = [x for tup in zip(*picked) for x in tup] if len(picked) > 1 else picked[0]
    batches = []
    for i in range(0, len(mixed), bsize):
        part = mixed[i:i + bsize]
        specs = [list(s) for s, _, _ in part]
        work = [w for _, w, _ in part]
        counts = [c for _, _, c in part]
        qs = gen_queries(g, [tuple(s) for s in specs], csr=csr)
        rs = engine.match_batch(qs, algo=ALGO_FUSED)
        if [int(r.count) for r in rs] != counts:
            raise RuntimeError("counts changed between selection and batching")
        hashes = [int(r.hash) for r in rs]
        sub = _ref_subset(work, ref_work, ref_query_work)
        batches.append(dict(specs=specs, work=work, counts=counts, hashes=[str(h) for h in hashes],
                            ref_subset=sub))
    m = dict(workload=name, graph=GRAPH_DESC[name], graph_digest=graph_digest(g), batch_size=bsize,
             work_budget=WORK_BUDGET, selection="first candidates of a seeded random-walk sequence whose "
             "heuristic-order enumeration examines at most work_budget driver entries",
             ref_subset_rule=f"per batch, in batch order, the queries with work <= {ref_query_work} until "
             f"their work adds up to {ref_work}",
             tune_specs=[list(s) for s, _, _ in tune], made_s=round(time.time() - t, 1), batches=batches)
    return m


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description="write workload manifests (needs a GPU)")
    ap.add_argument("--write", nargs="+", default=[], choices=["c1", "c2", "c4", "c5"])
    ap.add_argument("--out", default=str(MANIFESTS))
    ap.add_argument("--digests", action="store_true", help="print every workload graph's digest")
    args = ap.parse_args(argv)
    if args.digests:
        for n in NAMES:
            print(n, graph_digest(build_graph(n)), flush=True)
    if args.write:
        from . import Engine
        out = Path(args.out)
        out.mkdir(parents=True, exist_ok=True)
        with Engine(0, arena_bytes=64 << 30) as e:
            for n in args.write:
                m = make_manifest(e, n)
                (out / f"{n}.json").write_text(json.dumps(m, indent=0))
                print(f"{n}: {sum(len(b['specs']) for b in m['batches'])} queries, {m['made_s']} s", flush=True)


if __name__ == "__main__":
    main()
