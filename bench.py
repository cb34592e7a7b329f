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

Workloads (fsig_gb300/workloads.py): seeded synthetic graphs with the five
configurations' shapes; the queries of each workload are fixed by its
manifest (fsig_gb300/manifests/<name>.json), from which both arms rebuild
them with the host generators.

Order: the learned order (the packaged order-scoring network,
fsig_gb300/order_net.npy) when it exists, with a per-query work limit; a query
over the limit is carried into the next batch with its heuristic order
attached (the last ones run in a batch of their own), inside the timed region.
After the timed region the same batches run in heuristic order
("heuristic_batched") and every count and hash is compared between the two.
"single_query_path" is the plain one-query-per-call heuristic path
(fsig_match) on a sample.  Launch knobs are tuned on the manifest's tuning
batch, which is never timed.

Parity: cpu_baseline runs the CPU oracle on batch 0's reference subset (the
queries the CPU arm times) and compares every count and hash with the GPU's
results for the same queries ("oracle_check"); a mismatch fails the run.

--impl reference times the reference's matching semantics on the host
cores: the reference's matchers are GPU code with no CPU implementation, so
this arm runs the CPU backtracking port of them (oracle/) with all host
threads, on each step's reference subset -- the same queries the GPU arm
reports under "matched_subset".  It loads no library of the engine (its
generators come from oracle/build.py's copy).
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
from fsig_gb300 import workloads as W  # noqa: E402

METRIC = "queries/s & embeddings/s on 1 GB300, learned vs heuristic order, bit-exact"
PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0

# DRAM bytes (read + write) of one enumerate_kernel launch on a config-5
# batch, from an ncu capture (profiles/enumerate_kernel_c5.md: 648.4 MB/s over
# 392.1 ms); its loads are served from L2 at about 99 %.
ENUM_TRAFFIC_BYTES_PER_LAUNCH = 257_250_000


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def sig(x: float, digits: int = 6) -> float:
    """x rounded to `digits` significant digits."""
    return float(f"{x:.{digits}g}") if x else 0.0


def shared_config(w: W.Workload, world: int) -> dict:
    """The workload description both arms print (identical by construction)."""
    m = w.manifest
    return {"workload": w.name, "graph": w.desc, "queries_per_step": len(w.batches[0]),
            "batches": len(w.batches), "manifest": f"fsig_gb300/manifests/{w.name}.json",
            "selection": f"{m['selection']} ({m['work_budget']})",
            "reference_subset": m["ref_subset_rule"],
            "l2": "inputs larger than L2 (resident graph arrays > 129 MB)" if w.name == "c5" else
                  "graph fits L2; batches differ step to step",
            "parallelism": f"replicas x{world}, each rank runs the manifest's batches from batch <rank>"}


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
# the CPU oracle on a fixed subset of a batch (cpu_baseline, reference arm)
# ---------------------------------------------------------------------------
def oracle_on(w: W.Workload, queries, threads: int = 0) -> tuple:
    """(results [(count, hash)], seconds, threads): the oracle's backtracking
    matcher on the host cores (all of them unless threads is given), every
    query to completion."""
    from oracle import oracle as O  # the CPU legs only
    off, adj = w.csr
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    res = []
    for q in queries:
        c, h, _ = O.match(w.graph.labels, off, adj, q.labels, q.edges, threads=threads)
        res.append((int(c), int(h)))
    return res, time.perf_counter() - t0, threads


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
    t = time.time()
    w = W.load(args.workload, rank=dist.rank)
    batches = w.batches
    log(f"[bench] workload {w.name}: {sum(len(b) for b in batches)} queries in {len(batches)} batches from the "
        f"manifest, built in {time.time() - t:.1f}s")
    with F.Engine(dev, arena_bytes=args.arena_gb << 30) as e:
        e.load_graph(w.graph)
        log(f"[bench] graph resident: {e.graph_info()}")
        if order == "learned":
            e.mpnn_set_params(learn.load_params())
        limit = args.max_work or (W.WORK_BUDGET if order == "learned" else 0)

        use_graph = not args.no_graph
        knobs, tune_note = {}, "defaults"
        if not args.no_autotune:
            from fsig_gb300 import autotune
            t = time.time()
            osrc = F.ORDER_LEARNED if order == "learned" else F.ORDER_HEURISTIC
            knobs, trials = autotune.tune(e, w.tune, algo=algo, order_source=osrc, max_work=limit,
                                          use_graph=use_graph)
            tune_note = (f"coordinate descent on the manifest's tuning batch ({len(w.tune)} queries, never timed), "
                         f"{len(trials)} trials, {time.time() - t:.1f}s")
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
        nq = fallbacks = 0
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
        # every result against the manifest's record of the same query
        manifest_equal = all(results[k] == list(zip(w.counts[k % len(batches)], w.hashes[k % len(batches)]))
                             for k in range(args.steps))
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
        # the reference subsets (the queries the CPU arm times), one batch each
        sub_q = sub_emb = 0
        sub_dev = sub_wall = 0.0
        for k in range(len(batches)):
            qs = [batches[k][i] for i in w.ref_subset[k]]
            ts = time.perf_counter()
            rs = e.match_batch(qs, algo=algo, order_source=F.ORDER_HEURISTIC, use_graph=use_graph, **knobs)
            sub_wall += time.perf_counter() - ts
            st = e.last_stats()
            sub_dev += (st["ms_filter"] + st["ms_join"]) / 1e3
            sub_q += len(qs)
            sub_emb += sum(r.count for r in rs)
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
        "value": sig(value),
        "unit": "queries/s",
        "embeddings_per_s": sig(tot_emb / dev_s),
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": sig(dev_s * 1e3 / args.steps),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32",
        "data": "synthetic (seeded generators; no dataset available)",
        "config": shared_config(w, dist.world),
        "arm": {"algo": args.algo, "order": order, "work_limit": limit, "cuda_graph": use_graph,
                "knobs": knobs or "defaults", "autotune": tune_note, "learned_fallbacks": fallbacks,
                "results_equal_manifest": bool(manifest_equal)},
        "e2e": {"value": sig(tot_q / wall_s), "unit": "queries/s",
                "h2d_bytes_per_step": int(h2d / args.steps), "d2h_bytes_per_step": int(d2h / args.steps)},
        "heuristic_batched": {"value": sig(tot_q / heur_s), "unit": "queries/s",
                              "ms_per_step": sig(heur_s * 1e3 / args.steps),
                              "counts_and_hashes_identical": bool(identical),
                              "note": "the same batches in heuristic order, device time, after the timed region"},
        "latency_ms": {
            "batched_p50": round(1e3 * float(np.percentile(step_wall, 50)), 2),
            "batched_p99": round(1e3 * float(np.percentile(step_wall, 99)), 2),
            "single_p50": round(1e3 * float(np.percentile(single_lat, 50)), 2),
            "single_p99": round(1e3 * float(np.percentile(single_lat, 99)), 2),
            "note": "per query, wall clock: a batched query completes with its batch (call to results), a single "
                    "query with its own fsig_match call"},
        "single_query_path": {"value": sig(single_qps), "unit": "queries/s",
                              "sample": f"first {len(single)} queries of batch 0, one fsig_match call each (algo 2, "
                                        "reference-exact heuristic order), wall clock"},
        "matched_subset": {"queries": sub_q, "embeddings": sub_emb,
                           "gpu_device_qps": sig(sub_q / sub_dev), "gpu_e2e_qps": sig(sub_q / sub_wall),
                           "gpu_device_emb_per_s": sig(sub_emb / sub_dev),
                           "note": "each batch's reference subset (the queries the CPU arm times) as one batch, "
                                   "heuristic order; a few queries per batch, so launch-latency bound"},
        "gpu_launches": int(launches),
        "enumeration_passes": int(passes),
        "roofline": {"bound": "hbm", "kernel": "enumerate_kernel", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": "measured" if PEAKS.exists() else "fallback",
                     "traffic": ENUM_TRAFFIC_BYTES_PER_LAUNCH if args.workload == "c5" else None,
                     "traffic_note": ("DRAM bytes of one config-5 batch launch (ncu); requested bytes are "
                                      "served from L2 at about 99% hit: the kernel is issue-bound, not HBM-bound")
                                     if args.workload == "c5" else "no ncu capture of this workload",
                     "achieved_basis": "bytes requested by the kernel's global loads / kernel time, "
                                       + roof_basis},
        "clocks": clocks,
    }
    if dist.rank == 0 and not args.no_cpu_baseline:
        sub = w.ref_subset[0]
        qs = [batches[0][i] for i in sub]
        ores, cdt, threads = oracle_on(w, qs)
        gpu = [results[0][i] for i in sub]
        equal = ores == gpu
        cemb = sum(c for c, _ in ores)
        line["cpu_baseline"] = {"value": sig(len(qs) / cdt), "unit": "queries/s", "cores": threads, "kind": "port",
                                "embeddings_per_s": sig(cemb / cdt),
                                "sample": f"batch 0's reference subset: {len(qs)} queries ({cemb} embeddings), "
                                          f"oracle backtracking, {threads} threads, {cdt:.1f}s"}
        # the same oracle on one thread, over the subset's first query
        o1, t1, _ = oracle_on(w, qs[:1], threads=1)
        t1 = max(t1, 1e-9)
        line["cpu_baseline"]["single_thread"] = {
            "value": sig(1 / t1), "unit": "queries/s", "embeddings_per_s": sig(o1[0][0] / t1),
            "sample": f"the subset's first query ({o1[0][0]} embeddings), 1 thread, {t1:.1f}s"}
        line["oracle_check"] = {"queries": len(qs), "equal": bool(equal),
                                "note": "oracle (count, hash) against the timed step-0 results of the same queries"}
        line["matched_subset"]["cpu_qps_batch0"] = sig(len(qs) / cdt)
        line["matched_subset"]["cpu_emb_per_s_batch0"] = sig(cemb / cdt)
        if not equal:
            bad = [i for i, (a, b) in zip(sub, zip(ores, gpu)) if a != b]
            print(json.dumps(line), flush=True)
            raise SystemExit(f"oracle check failed on batch 0 queries {bad}")
    if not identical or not manifest_equal:
        print(json.dumps(line), flush=True)
        raise SystemExit("results differ between orders or from the manifest's record")
    return line


def run_reference(args, dist):
    if dist.rank != 0:
        return None
    from oracle import build as obuild
    F.use_generator_library(obuild.build_generators())
    t = time.time()
    w = W.load(args.workload)
    log(f"[reference] workload {w.name} built in {time.time() - t:.1f}s (generators from oracle/_build)")
    nb = len(w.batches)
    # warm-up: the first query of each step's subset
    for i in range(args.warmup):
        k = i % nb
        oracle_on(w, [w.batches[k][j] for j in w.ref_subset[k][:1]])
    done = emb = 0
    checked = mismatched = 0
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    step_s = []
    for k in range(args.steps):
        b = k % nb
        idx = w.ref_subset[b]
        res, dt, threads = oracle_on(w, [w.batches[b][j] for j in idx])
        step_s.append(dt)
        done += len(idx)
        emb += sum(c for c, _ in res)
        for j, r in zip(idx, res):
            checked += 1
            mismatched += r != (w.counts[b][j], w.hashes[b][j])
        log(f"[reference] step {k}: {len(idx)} queries of batch {b}, {dt:.2f}s")
    dt = time.perf_counter() - t0
    v = done / dt
    sample = (f"per step, the step's batch's reference subset ({min(len(s) for s in w.ref_subset)}-"
              f"{max(len(s) for s in w.ref_subset)} queries; the GPU arm's 'matched_subset' times the same "
              f"queries), oracle backtracking (the reference's matchers exist only as GPU code), {threads} threads")
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": sig(v),
        "unit": "queries/s",
        "embeddings_per_s": sig(emb / dt),
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": sig(dt * 1e3 / args.steps),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32",
        "data": "synthetic (seeded generators; no dataset available)",
        "config": shared_config(w, dist.world),
        "cpu_baseline": {"value": sig(v), "unit": "queries/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": sig(v), "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "oracle_vs_manifest": {"queries": checked, "mismatched": mismatched,
                               "note": "oracle (count, hash) against the engine's results recorded in the manifest"},
    }


def run_c3(args, dist):
    """Config 3 at full size (R-MAT 2^20 vertices / 2^24 edges, unlabeled):
    the five 5-vertex patterns.  Their embedding counts are about 1e15-1e16
    (a scale series shows them growing about 3.6x per doubling of the graph),
    so a whole pattern takes hours to days to enumerate.  Each step times one
    pattern over a stratified sample of its root tasks (fsig_match_range: the
    task space cut into `c3_strata` equal strata, one random range of
    `c3_tasks` tasks in each), giving measured throughput at full size and an
    estimate of the whole pattern's count and device time (the sum over strata
    of the stratum's size times its sample's mean per task)."""
    if dist.rank != 0:
        return None
    if args.c3_full:
        return run_c3_full(args, dist)
    g = W.build_graph("c3")
    rng = np.random.default_rng(33)
    names = list(W.PATTERNS)
    per = []
    with F.Engine(dist.local, arena_bytes=args.arena_gb << 30) as e:
        e.load_graph(g)
        with ClockSampler(dist.local) as clk:
            for k in range(args.steps + args.warmup):
                name = names[k % len(names)]
                q = W.pattern(name)
                _, T = e.match_range(q, F.ALGO_GSI, 0, 0)
                # warm-up steps sample a single stratum
                K = max(1, min(args.c3_strata if k >= args.warmup else 1, T))
                bounds = np.linspace(0, T, K + 1).astype(np.int64)
                cnt_est = time_est = 0.0
                s_cnt = s_work = 0
                s_ms = 0.0
                for j in range(K):
                    lo, hi = int(bounds[j]), int(bounds[j + 1])
                    if hi <= lo:
                        continue
                    t0 = int(rng.integers(lo, max(lo + 1, hi - args.c3_tasks + 1)))
                    t1 = min(hi, t0 + args.c3_tasks)
                    r, _ = e.match_range(q, F.ALGO_GSI, t0, t1)
                    st = e.last_stats()
                    ms = st["ms_join"] + st["ms_filter"]
                    scale = (hi - lo) / (t1 - t0)
                    cnt_est += scale * r.count
                    time_est += scale * ms / 1e3
                    s_cnt += r.count
                    s_work += st["enum_examines"] * 32
                    s_ms += ms
                if k >= args.warmup:
                    per.append({"pattern": name, "edges": [list(x) for x in W.PATTERNS[name]], "tasks_total": T,
                                "sampled_tasks": K * args.c3_tasks, "sampled_embeddings": s_cnt,
                                "sampled_device_s": round(s_ms / 1e3, 3),
                                "embeddings_per_s": sig(s_cnt / (s_ms / 1e3)) if s_ms else 0.0,
                                "driver_entries_per_s": sig(s_work / (s_ms / 1e3)) if s_ms else 0.0,
                                "estimated_count": sig(cnt_est, 3), "estimated_hours": sig(time_est / 3600, 3)})
                    log(f"[c3] {per[-1]}")
    tot_emb = sum(p["sampled_embeddings"] for p in per)
    tot_s = sum(p["sampled_device_s"] for p in per)
    return {
        "metric": "embeddings/s, unlabeled 5-vertex patterns at full size (sampled root tasks)",
        "value": sig(tot_emb / tot_s) if tot_s else 0.0, "unit": "embeddings/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sig(tot_s * 1e3 / max(len(per), 1)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded generators; no dataset available)",
        "config": {"workload": "c3", "graph": W.GRAPH_DESC["c3"],
                   "sample": f"{args.c3_strata} strata x {args.c3_tasks} root tasks per pattern, seeded"},
        "patterns": per, "clocks": clk.summary()}


def run_c3_full(args, dist):
    """One config-3 pattern over its whole task space at full size, in
    fsig_match_range pieces of root tasks -- one task first (the lowest ids
    are R-MAT's hubs, the heaviest roots), the piece doubled while a piece
    takes under 10 s, up to c3_piece: the exact count and hash when the whole
    space finishes within c3_budget_s seconds, else the part done."""
    g = W.build_graph("c3")
    q = W.pattern(args.c3_full)
    count = hsum = 0
    dev_s = 0.0
    with F.Engine(dist.local, arena_bytes=args.arena_gb << 30) as e:
        e.load_graph(g)
        _, T = e.match_range(q, F.ALGO_GSI, 0, 0)
        t0 = time.perf_counter()
        done = 0
        piece = 1
        with ClockSampler(dist.local) as clk:
            while done < T and time.perf_counter() - t0 < args.c3_budget_s:
                r, _ = e.match_range(q, F.ALGO_GSI, done, min(T, done + piece))
                st = e.last_stats()
                ms = st["ms_filter"] + st["ms_join"]
                dev_s += ms / 1e3
                count += r.count
                hsum = (hsum + r.hash) % (1 << 64)
                done = min(T, done + piece)
                log(f"[c3] {args.c3_full}: tasks {done}/{T} (piece {piece}, {ms / 1e3:.1f}s), {count} embeddings, "
                    f"{time.perf_counter() - t0:.0f}s")
                piece = min(args.c3_piece, piece * 2) if ms < 10e3 else max(1, piece // 2)
        wall = time.perf_counter() - t0
    complete = done >= T
    return {"metric": "embeddings/s, one unlabeled 5-vertex pattern at full size, every root task",
            "value": sig(count / dev_s) if dev_s else 0.0, "unit": "embeddings/s", "n_gpus": dist.world,
            "higher_is_better": True, "dtype": "u32", "data": "synthetic (seeded generators; no dataset available)",
            "config": {"workload": "c3", "graph": W.GRAPH_DESC["c3"], "pattern": args.c3_full,
                       "edges": [list(x) for x in W.PATTERNS[args.c3_full]], "max_piece_tasks": args.c3_piece},
            "complete": complete, "tasks_done": done, "tasks_total": T,
            "count": count if complete else None, "hash": hex(hsum) if complete else None,
            "count_so_far": count, "device_s": round(dev_s, 3), "wall_s": round(wall, 1), "clocks": clk.summary()}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="c5", choices=["c5", "c4", "c3", "c2", "c1"])
    ap.add_argument("--c3-strata", type=int, default=64, help="config 3: strata of each pattern's task space")
    ap.add_argument("--c3-tasks", type=int, default=4, help="config 3: root tasks sampled per stratum")
    ap.add_argument("--c3-full", default="", choices=[""] + list(W.PATTERNS),
                    help="config 3: enumerate this pattern over every root task instead of sampling")
    ap.add_argument("--c3-piece", type=int, default=16384, help="config 3 --c3-full: root tasks per call")
    ap.add_argument("--c3-budget-s", type=float, default=1800.0, help="config 3 --c3-full: time budget")
    ap.add_argument("--algo", default="fused", choices=["fsig", "gsi", "fused"])
    ap.add_argument("--order", default=None, choices=["heuristic", "learned"],
                    help="default: learned when the packaged network exists")
    ap.add_argument("--max-work", type=int, default=0,
                    help="per-query work limit (default: the selection budget in learned order, none otherwise)")
    ap.add_argument("--arena-gb", type=int, default=64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="ordinary launches instead of one CUDA graph per batch")
    ap.add_argument("--no-autotune", action="store_true", help="default launch knobs instead of autotuned ones")
    ap.add_argument("--single-sample", type=int, default=64)
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("at least 3 warm-up steps")
    dist = Dist()
    try:
        if args.workload == "c3":
            line = run_c3(args, dist) if args.impl == "ours" else {
                "impl": "reference", "unavailable": "config 3 patterns have ~1e15 embeddings each; the CPU oracle "
                "is timed on reduced-scale graphs of the same generator instead"}
        else:
            line = run_reference(args, dist) if args.impl == "reference" else run_ours(args, dist)
        if dist.rank == 0 and line is not None:
            print(json.dumps(line), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
