#!/usr/bin/env python3
"""Benchmark of the batched matching path: queries/s and embeddings/s on one
GB300 (whole job over N GPUs under torchrun), counts and hashes exact.

A step is one batch of queries (512 by default) matched against the resident
data graph through fsig_match_batch: filter + refinement + ordering + root
compaction + enumeration.

  value   queries / device time of the K timed batches (inputs resident: the
          data graph is loaded before timing; CUDA events on the engine's
          stream bracket each batch)
  e2e     the same metric through the C ABI call with host query buffers:
          wall time including packing, host->device copies of the query
          descriptors and device->host copies of the results

Order: the learned order (the packaged order-scoring network,
fsig_gb300/order_net.npy, trained on logs of the mid-scale graphs) when it
exists, with a per-query work limit; a query over the limit is carried into
the next batch with its heuristic order attached (the last ones run in a batch
of their own), inside the timed region.  After the timed region the same
batches run in heuristic order ("heuristic_batched"), and every count and
hash is compared between the two.  "single_query_path" is the plain
one-query-per-call heuristic path (fsig_match) on a sample.

Workloads (synthetic, seeded; no dataset is available):
  c5  Chung-Lu 2^22 vertices / 2^26 edges, exponent 2.0, seed 5, 32 Zipf
      labels; 2048 queries of 12-32 vertices, batches of 512 (default)
  c4  Chung-Lu 320,000 / 1,050,000, exponent 2.1, seed 2, 16 Zipf labels;
      4096 queries of 4-32 vertices, half dense half sparse, batches of 512
  c2  the c4 graph; 200 queries of 8 vertices (100 dense, 100 sparse)
  c1  R-MAT 10,000 / 50,000, seed 1, 8 uniform labels; 100 queries of 4

--impl reference times the reference's matching semantics on the host
cores: the reference's matchers are GPU code with no CPU implementation, so
this arm runs the CPU backtracking port of them (oracle/) with all host
threads, each step a bounded sample of the step's batch.
"""
from __future__ import annotations

import argparse
import json
import os
import signal
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import fsig_gb300 as F  # noqa: E402

METRIC = "queries/s & embeddings/s on 1 GB300, learned vs heuristic order, bit-exact"
PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0

# DRAM bytes per enumeration launch from an ncu capture; None until measured.
# DRAM bytes (read + write) of one enumerate_kernel launch on a heavy
# config-5 batch (about 5.4e8 driver windows), from an ncu capture
# (profiles/enumerate_kernel_c5.md); its loads are served from L2 at 98.9%.
ENUM_TRAFFIC_BYTES_PER_LAUNCH = 286_300_000


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def build_graph(name):
    if name == "c5":
        lab = F.gen_labels(1 << 22, 32, "zipf", seed=5)
        return F.gen_chung_lu(1 << 22, 1 << 26, 2.0, seed=5, labels=lab), "Chung-Lu 2^22 V / 2^26 E, exp 2.0, 32 Zipf labels"
    if name in ("c4", "c2"):
        lab = F.gen_labels(320000, 16, "zipf", seed=2)
        return F.gen_chung_lu(320000, 1050000, 2.1, seed=2, labels=lab), "Chung-Lu 320k V / 1.05M E, exp 2.1, 16 Zipf labels"
    if name == "c1":
        lab = F.gen_labels(10000, 8, "uniform", seed=1)
        return F.gen_rmat(10000, 50000, 0.57, 0.19, 0.19, seed=1, labels=lab), "R-MAT 10k V / 50k E, 8 uniform labels"
    raise SystemExit(f"unknown workload {name}")


# Candidate queries are random-walk extractions in a seeded sequence; a
# workload keeps, in order, the first ones whose enumeration under the
# heuristic order examines at most WORK_BUDGET driver entries (a property of
# query and graph alone, so the choice is the same on every run).  Walks are
# confined to the less frequent Zipf labels: over all labels, 12-32-vertex
# queries on the 2^22-vertex graph have more than 10^9 partial embeddings
# (none of 512 candidates fitted 2^26 examined entries).
WORK_BUDGET = 1 << 26


def candidate_specs(name, rank):
    rng = np.random.default_rng(1000 + rank)
    base = 1_000_000 * (rank + 1)
    if name == "c5":
        # 2048 dense queries of 12-32 vertices on labels >= 8, batches of 512
        sizes = rng.integers(12, 33, 32768)
        return [[(int(n), F.QUERY_DENSE, base + i, 8) for i, n in enumerate(sizes)]], [2048], 512
    if name == "c4":
        # 4096 queries of 4-32 vertices, half dense half sparse, labels >= 4
        sizes = rng.integers(4, 33, 32768)
        dense = [(int(n), F.QUERY_DENSE, base + i, 4) for i, n in enumerate(sizes)]
        sparse = [(int(n), F.QUERY_SPARSE, base + 500_000 + i, 4) for i, n in enumerate(sizes)]
        return [dense, sparse], [2048, 2048], 512
    if name == "c2":
        dense = [(8, F.QUERY_DENSE, base + i, 4) for i in range(4096)]
        sparse = [(8, F.QUERY_SPARSE, base + 500_000 + i, 4) for i in range(4096)]
        return [dense, sparse], [100, 100], 200
    if name == "c1":
        return [[(4, F.QUERY_INDUCED, base + i) for i in range(100)]], [100], 100
    raise SystemExit(f"unknown workload {name}")


def make_workload(name, rank, engine):
    """Graph (loaded into the engine) and the selected query batches."""
    t = time.time()
    g, gdesc = build_graph(name)
    csr = g.csr()
    engine.load_graph(g)
    pools, wants, batch = candidate_specs(name, rank)
    qs = []
    for pool, want in zip(pools, wants):
        picked = []
        for i in range(0, len(pool), 2048):  # generate candidates in slices, select, stop when enough
            cand = F.gen_queries(g, pool[i:i + 2048], csr=csr)
            picked += F.select_within_budget(engine, cand, want - len(picked), WORK_BUDGET)
            if len(picked) >= want:
                break
        if len(picked) < want:
            raise SystemExit(f"workload {name}: only {len(picked)} of {want} candidates fit the work budget")
        qs.append(picked)
    # interleave the pools so that every batch has the same mix
    mixed = [q for tup in zip(*qs) for q in tup] if len(qs) > 1 else qs[0]
    batches = [mixed[i:i + batch] for i in range(0, len(mixed), batch)]
    log(f"[bench] workload {name}: {len(mixed)} queries in {len(batches)} batches, setup {time.time() - t:.1f}s")
    return g, csr, gdesc, batches


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.send_signal(signal.SIGTERM)
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]) if parts[3] not in ("[N/A]", "N/A") else 0.0,
                             parts[5], parts[6], parts[7], parts[8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[3:]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": reasons}


# ---------------------------------------------------------------------------
# distributed plumbing (torchrun); no data-path collective
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def cuda_sync():
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.synchronize()
    except ImportError:
        pass


# ---------------------------------------------------------------------------
# CPU baseline: the oracle port on the host cores, bounded sample
# ---------------------------------------------------------------------------
def cpu_sample(g, csr, queries, budget_s):
    from oracle import oracle as O  # the CPU leg only
    off, adj = csr
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    done = emb = 0
    for q in queries:
        c, h, _ = O.match(g.labels, off, adj, q.labels, q.edges, threads=threads)
        done += 1
        emb += c
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return done, emb, dt, threads


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------
class StepStats:
    """Device time and traffic of the engine calls one arm makes."""

    def __init__(self):
        self.dev_ms = self.enum_ms = 0.0
        self.enum_bytes = self.launches = self.h2d = self.d2h = self.passes = 0
        self.enum_timed = True

    def add(self, st):
        self.dev_ms += st["ms_filter"] + st["ms_join"]
        if st["ms_enum"] < 0:
            self.enum_timed = False
        self.enum_ms += max(st["ms_enum"], 0.0)
        self.enum_bytes += st["enum_bytes"]
        self.launches += st["kernel_launches"]
        self.passes += st["enum_passes"]
        self.h2d += st["h2d_bytes"]
        self.d2h += st["d2h_bytes"]


def run_ours(args, dist):
    from fsig_gb300 import learn
    dev = dist.local
    algo = {"fsig": F.ALGO_FSIG, "gsi": F.ALGO_GSI, "fused": F.ALGO_FUSED}[args.algo]
    order = args.order or ("learned" if learn.WEIGHTS.exists() else "heuristic")
    with F.Engine(dev, arena_bytes=args.arena_gb << 30) as e:
        g, csr, gdesc, batches = make_workload(args.workload, dist.rank, e)
        info = e.graph_info()
        log(f"[bench] graph resident: {info}")
        if order == "learned":
            e.mpnn_set_params(learn.load_params())
        limit = args.max_work or (WORK_BUDGET if order == "learned" else 0)

        use_graph = not args.no_graph
        knobs, tune_note = {}, "defaults"
        if not args.no_autotune:
            from fsig_gb300 import autotune
            t = time.time()
            osrc = F.ORDER_LEARNED if order == "learned" else F.ORDER_HEURISTIC
            knobs, trials = autotune.tune(e, batches[-1], algo=algo, order_source=osrc, max_work=limit,
                                          use_graph=use_graph)
            tune_note = f"coordinate descent on the last batch, {len(trials)} trials, {time.time() - t:.1f}s"
            log(f"[bench] autotuned {knobs} ({tune_note})")

        feed = learn.LearnedFeed(e, algo, limit, use_graph=use_graph, **knobs) if order == "learned" else None

        def step(k, b, acc, results):
            if feed:
                return feed.step(k, b, results, acc.add)
            rs = e.match_batch(b, algo=algo, order_source=F.ORDER_HEURISTIC, max_work=limit, use_graph=use_graph,
                               **knobs)
            acc.add(e.last_stats())
            results[k] = [(r.count, r.hash) for r in rs]
            return rs, 0

        warm = [None] * args.warmup
        for i in range(args.warmup):
            step(i, batches[i % len(batches)], StepStats(), warm)
        if feed:
            feed.flush(warm)
        dist.barrier()
        cuda_sync()
        acc = StepStats()
        nq = over = fallbacks = 0
        results = [None] * args.steps
        with ClockSampler(dev) as clk:
            t0 = time.perf_counter()
            step_wall = []
            for k in range(args.steps):
                b = batches[k % len(batches)]
                before = acc.dev_ms
                ts = time.perf_counter()
                rs, fb = step(k, b, acc, results)
                step_wall.append(time.perf_counter() - ts)
                nq += len(b)
                fallbacks += fb
                st = e.last_stats()
                log(f"[bench] step {k}: {len(b)} queries, {sum(r.count for r in rs)} embeddings, device "
                    f"{acc.dev_ms - before:.2f} ms ({order} order, {fb} fallbacks); last call: filter "
                    f"{st['ms_filter']:.2f} ms, join {st['ms_join']:.2f} ms (enumeration {st['ms_enum']:.2f} ms, "
                    f"{st['enum_passes']} passes); tasks {st['enum_tasks']} pops {st['enum_pops']} handoffs "
                    f"{st['enum_handoffs']} records {st['enum_records']} examines {st['enum_examines']}")
            if feed:
                feed.flush(results, acc.add)
            cuda_sync()
            wall = time.perf_counter() - t0
        dist.barrier()
        emb = sum(c for step_res in results for c, _ in step_res)
        # the same batches in heuristic order: the comparison and the bit-exactness check
        heur = StepStats()
        identical = True
        for k in range(args.steps):
            b = batches[k % len(batches)]
            rs = e.match_batch(b, algo=algo, order_source=F.ORDER_HEURISTIC, use_graph=use_graph, **knobs)
            heur.add(e.last_stats())
            identical &= [(r.count, r.hash) for r in rs] == results[k]
        dev_ms, enum_ms, enum_bytes = acc.dev_ms, acc.enum_ms, acc.enum_bytes
        roof_basis = "timed batches"
        if not acc.enum_timed:
            # kernel time inside a graph was not measurable: the roofline comes
            # from the same batches launched without a graph
            roof = StepStats()
            for k in range(args.steps):
                b = batches[k % len(batches)]
                e.match_batch(b, algo=algo, order_source=F.ORDER_LEARNED if order == "learned" else F.ORDER_HEURISTIC,
                              max_work=limit, use_graph=False, **knobs)
                roof.add(e.last_stats())
            enum_ms, enum_bytes = roof.enum_ms, roof.enum_bytes
            roof_basis = "the timed batches again, launched without a graph"
        launches, h2d, d2h, passes = acc.launches, acc.h2d, acc.d2h, acc.passes
        # the plain single-query path (fsig_match, heuristic order) on a sample
        single = batches[0][: args.single_sample]
        t1 = time.perf_counter()
        single_lat = []
        for q in single:
            ts = time.perf_counter()
            e.match(q, F.ALGO_GSI)
            single_lat.append(time.perf_counter() - ts)
        single_qps = len(single) / (time.perf_counter() - t1)
    clocks = clk.summary()
    heur_s = dist.max(heur.dev_ms / 1e3)
    dev_s = dist.max(dev_ms / 1e3)
    wall_s = dist.max(wall)
    tot_q = dist.sum(nq)
    tot_emb = dist.sum(emb)
    value = tot_q / dev_s
    peaks = json.loads(PEAKS.read_text()) if PEAKS.exists() else {}
    peak = peaks.get("hbm_gbs", FALLBACK_HBM_GBS)
    achieved = (enum_bytes / (enum_ms / 1e3)) / 1e9 if enum_ms > 0 else 0.0
    line = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "queries/s",
        "embeddings_per_s": round(tot_emb / dev_s, 1),
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(dev_s * 1e3 / args.steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32",
        "data": "synthetic (seeded generators; no dataset available)",
        "config": {"workload": args.workload, "graph": gdesc, "queries_per_step": len(batches[0]),
                   "algo": args.algo, "order": order, "parallelism": f"replicas x{dist.world}, queries sharded",
                   "l2": "inputs larger than L2 (resident graph arrays > 129 MB)" if args.workload in ("c5",) else
                   "graph fits L2; batches differ step to step",
                   "work_limit": limit, "cuda_graph": use_graph, "knobs": knobs or "defaults",
                   "autotune": tune_note, "queries_over_limit": over, "learned_fallbacks": fallbacks,
                   "selection": f"first queries of a seeded random-walk sequence whose enumeration examines at most "
                                f"{WORK_BUDGET} driver entries"},
        "e2e": {"value": round(tot_q / wall_s, 3), "unit": "queries/s",
                "h2d_bytes_per_step": int(h2d / args.steps), "d2h_bytes_per_step": int(d2h / args.steps)},
        "heuristic_batched": {"value": round(tot_q / heur_s, 3), "unit": "queries/s",
                              "ms_per_step": round(heur_s * 1e3 / args.steps, 3),
                              "counts_and_hashes_identical": bool(identical),
                              "note": "the same batches in heuristic order, device time, after the timed region"},
        "latency_ms": {
            "batched_p50": round(1e3 * float(np.percentile(step_wall, 50)), 2),
            "batched_p99": round(1e3 * float(np.percentile(step_wall, 99)), 2),
            "single_p50": round(1e3 * float(np.percentile(single_lat, 50)), 2),
            "single_p99": round(1e3 * float(np.percentile(single_lat, 99)), 2),
            "note": "per query, wall clock: a batched query completes with its batch (call to results), a single "
                    "query with its own fsig_match call"},
        "single_query_path": {"value": round(single_qps, 3), "unit": "queries/s",
                              "sample": f"first {len(single)} queries of batch 0, one fsig_match call each (algo 2, "
                                        "reference-exact heuristic order), wall clock"},
        "gpu_launches": int(launches),
        "enumeration_passes": int(passes),
        "roofline": {"bound": "hbm", "kernel": "enumerate_kernel", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": "measured" if PEAKS.exists() else "fallback",
                     "traffic": ENUM_TRAFFIC_BYTES_PER_LAUNCH if args.workload == "c5" else None,
                     "traffic_note": ("DRAM bytes of one heavy config-5 batch launch (ncu); requested bytes are "
                                      "served from L2 at 98.9% hit: the kernel is issue-bound, not HBM-bound")
                                     if args.workload == "c5" else "no ncu capture of this workload",
                     "achieved_basis": "bytes requested by the kernel's global loads / kernel time, "
                                       + roof_basis},
        "clocks": clocks,
    }
    if dist.rank == 0 and not args.no_cpu_baseline:
        done, cemb, cdt, threads = cpu_sample(g, csr, batches[0], args.cpu_budget)
        line["cpu_baseline"] = {"value": round(done / cdt, 3), "unit": "queries/s", "cores": threads, "kind": "port",
                                "sample": f"first {done} queries of batch 0 ({cemb} embeddings), oracle backtracking, "
                                          f"{threads} threads, {cdt:.1f}s"}
    return line


def run_reference(args, dist):
    if dist.rank != 0:
        return None
    # The workload's queries are chosen with the GPU engine (a property of
    # query and graph); the timed work below runs only on the host cores.
    with F.Engine(dist.local, arena_bytes=args.arena_gb << 30) as e:
        g, csr, gdesc, batches = make_workload(args.workload, 0, e)
    per_step = max(1.0, args.ref_step_s)
    for i in range(args.warmup):
        cpu_sample(g, csr, batches[i % len(batches)], per_step / 4)
    done_tot = emb_tot = 0
    t0 = time.perf_counter()
    threads = os.cpu_count() or 1
    for k in range(args.steps):
        done, emb, dt, threads = cpu_sample(g, csr, batches[k % len(batches)], per_step)
        done_tot += done
        emb_tot += emb
    dt = time.perf_counter() - t0
    v = done_tot / dt
    sample = (f"per step: the first queries of the step's batch until {per_step:.0f}s, oracle backtracking "
              f"(the reference's matchers exist only as GPU code), {threads} threads")
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": round(v, 3),
        "unit": "queries/s",
        "embeddings_per_s": round(emb_tot / dt, 1),
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(dt * 1e3 / args.steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32",
        "data": "synthetic (seeded generators; no dataset available)",
        "config": {"workload": args.workload, "graph": gdesc, "queries_per_step": len(batches[0])},
        "cpu_baseline": {"value": round(v, 3), "unit": "queries/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(v, 3), "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="c5", choices=["c5", "c4", "c2", "c1"])
    ap.add_argument("--algo", default="fused", choices=["fsig", "gsi", "fused"])
    ap.add_argument("--order", default=None, choices=["heuristic", "learned"],
                    help="default: learned when the packaged network exists")
    ap.add_argument("--max-work", type=int, default=0,
                    help="per-query work limit (default: the selection budget in learned order, none otherwise)")
    ap.add_argument("--arena-gb", type=int, default=64)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--ref-step-s", type=float, default=8.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="ordinary launches instead of one CUDA graph per batch")
    ap.add_argument("--no-autotune", action="store_true", help="default launch knobs instead of autotuned ones")
    ap.add_argument("--single-sample", type=int, default=64)
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("at least 3 warm-up steps")
    dist = Dist()
    try:
        line = run_reference(args, dist) if args.impl == "reference" else run_ours(args, dist)
        if dist.rank == 0 and line is not None:
            print(json.dumps(line), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
