#!/usr/bin/env python
"""Benchmark of the neighbour-sampling estimator hot path on GB300.

Workload (default "rmat20"): undirected R-MAT scale 20, edge factor 3, a/b/c/d = .57/.19/.19/.05,
self-loops and duplicates removed (~3.1M edges, seeded synthetic input); one step = the
triangle, 4-clique, 3-chain and 4-chain estimators with 2^26 samples each (2^28 estimators).

  value : samples/s over the timed steps, device time from CUDA events on the launching stream
          (graph resident in HBM; L2 flushed between steps by writing a 512 MiB buffer).
  e2e   : samples/s through the public API (ZGraphInstance.calculate -> zg_run): host wall time
          per query including the device->host read of each result.
  roofline: dominant kernel, algorithmic bytes = access-model sectors x 32 B per sample (measured
          per program by the debug kernel on 2^16 samples) x samples / kernel time.
  cpu_baseline: the CPU restatement of the reference path (oracle, all host threads) on a
          bounded sample of the same workload.

--impl reference runs that CPU restatement as the measured arm (the reference is CPU code and
does not build on this host without its MPI/NUMA stack).  Under torchrun each rank runs its
own shard of sample indices (weak scaling); rank 0 prints one JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sampling-graph-mining_gb300"))

METRIC = "time-to-1%-error@95% and samples/s, learned vs plain ELP, 1 GB300"
WORKLOADS = {
    "rmat20": {"scale": 20, "edge_factor": 3, "a": 0.57, "b": 0.19, "c": 0.19, "seed": 1, "samples": 1 << 26,
               "programs": ["triangle", "four_clique", "three_chain", "four_chain"]},
    "rmat13": {"scale": 13, "edge_factor": 12, "a": 0.57, "b": 0.19, "c": 0.19, "seed": 1, "samples": 1 << 20,
               "programs": ["triangle"]},
}
# Batched workloads (one submit of many queries per step; graphs generated on the device):
#   chunglu_batch: Chung-Lu 4.8 M vertices, exponent 2.3, ~43 M edges, edge data in [0, 100);
#                  512 queries over {triangle, 3-motif, all-predicate w >= T, at-least-one w >= T},
#                  T uniform in [10, 90], budgets 2^U(12, 24).
#   rmat26:        R-MAT scale 26, edge factor 24 (~1.4 G edges); 4-clique, 5-star, 5-house at 2^30.
BATCH_WORKLOADS = {
    "chunglu_batch": {"gen": "chung_lu", "n": 4800000, "exponent": 2.3, "avg_degree": 18.0, "seed": 2024,
                      "max_weight": 100, "queries": 512},
    "rmat26": {"gen": "rmat", "scale": 26, "edge_factor": 24, "seed": 26, "samples": 1 << 30},
}
PROG_IDS = {"triangle": 1, "four_clique": 2, "three_chain": 3, "four_chain": 4}
EXACT_IDS = {"triangle": 1, "three_chain": 2, "four_chain": 3, "four_clique": 5}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="rmat20", choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-time-to-bound", action="store_true")
    ap.add_argument("--variants", default=None,
                    help="fixed launch shapes instead of tuning, e.g. triangle=4,four_clique=3 "
                         "(profiling runs: no tuner probe launches)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) > 8 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic(samples):
    """DRAM bytes (read + write) per launch of each sampling kernel from the committed ncu summary
    (profiles/k_sample_traffic_rmat20.txt), scaled to `samples` per launch; {} if absent."""
    out = {}
    try:
        with open(os.path.join(ROOT, "profiles", "k_sample_traffic_rmat20.txt")) as f:
            for line in f:
                if line.startswith("#") or not line.strip():
                    continue
                name, b, n = line.split()
                out[name] = float(b) * samples / float(n)
    except (OSError, ValueError):
        return {}
    return out


def l2_read_gbs(Z, mib=48, reps=100):
    """Read bandwidth of a 48 MiB buffer resident in the 129 MB L2 (zg_read_bandwidth: one
    persistent grid, CUDA events): the L2 view of the roofline for graphs that nearly fit in L2."""
    return Z.read_bandwidth(mib << 20, reps)


def make_graph(Z, wl):
    e = Z.gen_rmat(wl["scale"], wl["edge_factor"], wl["a"], wl["b"], wl["c"], wl["seed"])
    return e, 1 << wl["scale"]


def cpu_baseline(wl, edges, nv, threads, target_s=12.0):
    """The oracle (CPU restatement of the reference path) on a bounded sample of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    og = O.OracleGraph(edges, nv)
    rates, total_samples, total_s = {}, 0, 0.0
    budget = target_s / len(wl["programs"])
    for name in wl["programs"]:
        prog = O.OracleProgram(PROG_IDS[name])
        n = 1 << 14
        while True:
            t0 = time.perf_counter()
            O.run(og, prog, n, 0, 17, PROG_IDS[name], threads)
            dt = time.perf_counter() - t0
            if dt > budget / 4 or n >= (1 << 26):
                break
            n *= 4
        rates[name] = n / dt
        total_samples += n
        total_s += dt
    return {"value": total_samples / total_s, "unit": "samples/s", "cores": threads, "kind": "port",
            "sample": "%s: %d samples per pattern class (bounded), oracle/zg_oracle.c with %d threads; per pattern %s"
                      % (",".join(wl["programs"]), total_samples // len(wl["programs"]), threads,
                         {k: round(v) for k, v in rates.items()})}


def time_to_bound(Z, g, names, acc, eps=0.01, conf=0.95, cap=1 << 37, coverage_queries=40):
    """Time from query submission (graph resident) to an answer whose empirical 95 % half-width is
    <= 1 % of the estimate: plain ErrorProfile sizing vs the learned network, same bound check (zg_query).
    For 4-cliques the unbiased canonical-path program runs: the reference's estimator is biased (it
    finds ~60 % of the cliques), so a tight interval around it is not an accuracy claim."""
    import elp_learn as EL
    model = os.path.join(ROOT, "sampling-graph-mining_gb300", "elp_mlp.npz")
    if not os.path.exists(model):
        return {"skipped": "no trained network at %s" % model}
    net = Z.Mlp.load(model)
    out = {"eps": eps, "confidence": conf, "max_samples": cap, "model": "sampling-graph-mining_gb300/elp_mlp.npz",
           "patterns": {}}
    for name in names:
        prog_name = "four_clique_unbiased" if name == "four_clique" else name
        r = EL.compare(net, g, prog_name, eps=eps, conf=conf, seed=31, max_samples=cap)
        ex = acc[name]["exact"]
        for k in ("plain", "learned"):
            r[k]["rel_err_vs_exact"] = abs(r[k]["estimate"] - ex) / ex
        r["speedup_learned_over_plain"] = r["plain"]["seconds"] / r["learned"]["seconds"]
        out["patterns"][prog_name] = r
    # delivered accuracy: triangle queries over independent seeds, learned sizing + bound check
    prog = Z.Program(1)
    ex = acc["triangle"]["exact"] if "triangle" in acc else g.exact_count(1)
    inside, met = 0, 0
    for s in range(coverage_queries):
        q = Z.learned_query(net, g, prog, eps, conf, 1000 + s, 5000 + s, stream_id=0x60 + s, max_samples=cap)[0]
        met += q.bound_met
        inside += abs(q.estimate - ex) <= eps * ex
    out["coverage"] = {"pattern": "triangle", "queries": coverage_queries, "bound_met": met,
                       "within_1pct_of_exact": inside}
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    wl = WORKLOADS[args.workload]
    import zgraph as Z
    edges, nv = make_graph(Z, wl)
    threads = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    og = O.OracleGraph(edges, nv)
    progs = [(PROG_IDS[p], O.OracleProgram(PROG_IDS[p])) for p in wl["programs"]]
    # calibrate a bounded per-step sample (about 1-2 s of CPU per step)
    n = 1 << 12
    while True:
        t0 = time.perf_counter()
        for pid, p in progs:
            O.run(og, p, n, 0, 5, pid, threads)
        dt = time.perf_counter() - t0
        if dt > 0.5 or n >= wl["samples"]:
            break
        n *= 2
    for i in range(args.warmup):
        for pid, p in progs:
            O.run(og, p, n, i * n, 5, pid, threads)
    t0 = time.perf_counter()
    for i in range(args.steps):
        for pid, p in progs:
            O.run(og, p, n, (args.warmup + i) * n, 5, pid, threads)
    dt = time.perf_counter() - t0
    value = len(progs) * n * args.steps / dt
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1000 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int64/f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "%s: R-MAT scale %d ef %d (%d edges), %s; bounded sample %d per pattern per step"
                       % (args.workload, wl["scale"], wl["edge_factor"], len(edges), "+".join(wl["programs"]), n)},
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads, "kind": "port",
                             "sample": "%d samples x %d patterns per step, oracle/zg_oracle.c" % (n, len(progs))},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import zgraph as Z
    Z.init(local)
    wl = WORKLOADS[args.workload]
    n = wl["samples"]
    edges, nv = make_graph(Z, wl)
    t0 = time.perf_counter()
    g = Z.Graph.from_edges(edges, nv)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    names = wl["programs"]
    progs = [Z.Program(PROG_IDS[p]) for p in names]
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    # autotuner: pick each program's launch shape on this graph (setup, untimed)
    tuning = {}
    fixed = dict(kv.split("=") for kv in args.variants.split(",")) if args.variants else None
    for name, p in zip(names, progs):
        if fixed is not None:
            if name in fixed:
                p.set_variant(int(fixed[name]))
            tuning[name] = dict(p.variant(), fixed=True)
            continue
        best, ms = p.tune(g, 1 << 23, cuda_stream=sp)
        tuning[name] = {"variant": best, "min_blocks": p.variant()["min_blocks"], "grid": p.variant()["grid"],
                        "ms_per_variant_2^23": [round(x, 3) for x in ms]}
    d_res = torch.zeros((len(progs), Z.ZG_RESULT_BYTES if hasattr(Z, "ZG_RESULT_BYTES") else 112),
                        dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    seed = 20250101

    def enqueue(step, evs=None):
        for j, p in enumerate(progs):
            if evs is not None:
                evs[j].record(stream)
            p.run_async(g, n, seed, d_res[j].data_ptr(), stream_id=j + 1,
                        first_sample=(step * world + rank) * n, cuda_stream=sp)
        if evs is not None:
            evs[len(progs)].record(stream)

    for i in range(args.warmup):
        enqueue(i)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    per_prog = [0.0] * len(progs)
    step_ms = []
    for i in range(args.steps):
        flush.zero_()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(len(progs) + 1)]
        enqueue(args.warmup + i, evs)
        torch.cuda.synchronize()
        for j in range(len(progs)):
            per_prog[j] += evs[j].elapsed_time(evs[j + 1])
        step_ms.append(evs[0].elapsed_time(evs[-1]))
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * len(progs) * n * args.steps / (total_ms / 1000.0)
    res = [p.result_to_counters(bytes(d_res[j].cpu().numpy())) for j, p in enumerate(progs)]
    if world > 1:  # exact merge of the ranks' shards (integer limbs, no floating reduction)
        res = [Z.allgather_counters(r) for r in res]

    # end to end through the public API: calculate() per program, results read back each query
    # (each rank its own Philox streams, so the ranks draw different samples)
    insts = [getattr(Z, c)(g, seed=seed + 7, stream_id=16 * rank + j + 11) for j, c in
             enumerate({"triangle": "TriangleCountingInstance", "four_clique": "FourCliqueCountingInstance",
                        "three_chain": "ThreeChainCountingInstance",
                        "four_chain": "FourChainCountingInstance"}[p] for p in names)]
    for inst in insts:
        inst.calculate(n, 3, Z.Estimation())
    torch.cuda.synchronize()
    e2e_steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        for inst in insts:
            inst.calculate(n, 3, Z.Estimation())
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": world * len(insts) * n * e2e_steps / e2e_s, "unit": "samples/s", "h2d_bytes_per_step": 0,
           "d2h_bytes_per_step": len(insts) * 112}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    # algorithmic bytes per sample: access model from the debug kernel (2^16 samples)
    model, closures = {}, {}
    for j, p in enumerate(progs):
        tr = p.run_debug(g, 1 << 16, seed, stream_id=j + 1)
        model[names[j]] = float(tr["sectors"].mean()) * 32.0
        closures[names[j]] = float(tr["closures"].mean())  # conditional_close look-ups per sample
    peak, peak_kind = peaks()
    kern = []
    for j, name in enumerate(names):
        t = per_prog[j] / args.steps / 1000.0
        ach = model[name] * n / t / 1e9
        kern.append({"kernel": "k_sample<%s>" % name, "ms": per_prog[j] / args.steps, "bytes_per_sample": model[name],
                     "achieved_gbs": ach, "samples_per_s": n / t,
                     "closure_checks_per_sample": closures[name], "closure_checks_per_s": closures[name] * n / t,
                     "hits": int(res[j].hits), "estimate": res[j].estimate})
    dom = max(kern, key=lambda k: k["ms"])
    traffic = profile_traffic(n).get(dom["kernel"]) if args.workload == "rmat20" else None
    l2_gbs = l2_read_gbs(Z)
    # the DRAM bytes the kernel really moved (ncu, per launch) over its CUDA-event time: how close to
    # the HBM roof it runs, next to the access-model view above
    dram = {"gbs": traffic / (dom["ms"] / 1000.0) / 1e9, "frac": traffic / (dom["ms"] / 1000.0) / 1e9 / peak,
            "source": "traffic (ncu dram__bytes_read + write per launch) / measured kernel time"} if traffic else None
    roofline = {"bound": "hbm", "achieved": dom["achieved_gbs"], "peak": peak, "unit": "GB/s",
                "frac": dom["achieved_gbs"] / peak, "traffic": traffic, "dram": dram, "kernel": dom["kernel"],
                "l2": {"peak": l2_gbs, "frac": dom["achieved_gbs"] / l2_gbs if l2_gbs else None,
                       "peak_source": "measured live: reads of a 48 MiB buffer resident in L2 (zg_read_bandwidth)"},
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "per_kernel": kern}
    # accuracy against the GPU exact counts
    acc = {}
    for j, name in enumerate(names):
        ex = g.exact_count(EXACT_IDS[name])
        acc[name] = {"exact": ex, "estimate": res[j].estimate,
                     "rel_err": abs(res[j].estimate - ex) / ex if ex else None}
        if name == "four_clique":  # the reference's estimator is biased; the canonical-path one is not
            u = Z.Program(Z.PROG_FOUR_CLIQUE_UNBIASED).run(g, n, seed, stream_id=j + 1)
            acc["four_clique_unbiased"] = {"exact": ex, "estimate": u.estimate,
                                           "rel_err": abs(u.estimate - ex) / ex if ex else None}
    ttb = time_to_bound(Z, g, names, acc) if not args.no_time_to_bound else None
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int64/u192 exact (f64 reference 1/p)",
            "data": "synthetic (seeded R-MAT, zg_gen_rmat)",
            "config": {"workload": "%s: R-MAT scale %d, edge factor %d, a/b/c=.57/.19/.19, %d undirected edges; "
                                   "%s x 2^%d samples per step" % (args.workload, wl["scale"], wl["edge_factor"],
                                                                   len(edges), "+".join(names),
                                                                   n.bit_length() - 1),
                       "l2": "flushed between steps (512 MiB write)", "graph_build_s": round(build_s, 3),
                       "graph_device_bytes": int(g.meta().device_bytes), "launch_tuning": tuning},
            "e2e": e2e, "gpu_launches": 2 * len(progs) * args.steps, "clocks": clk, "roofline": roofline,
            "accuracy": acc, "time_to_bound": ttb}
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(wl, edges, nv, os.cpu_count() or 1)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def batch_queries(Z, rng, nq):
    """The Chung-Lu batched workload's queries; an at-least-one-predicate query is two batch
    queries (all triangles, and triangles of the w < T graph) whose estimates are subtracted."""
    qs = []
    for i in range(nq):
        kind = int(rng.integers(4))
        n = int(2 ** rng.uniform(12, 24))
        t = int(rng.integers(10, 91))
        seed = int(rng.integers(1, 1 << 40))
        if kind == 0:
            qs.append({"kind": Z.PROG_TRIANGLE, "n": n, "seed": seed, "stream_id": i})
        elif kind == 1:
            qs.append({"kind": Z.QUERY_THREE_MOTIF, "n": n, "seed": seed, "stream_id": 2 * i})
        elif kind == 2:
            qs.append({"kind": Z.PROG_TRIANGLE, "n": n, "seed": seed, "pred_op": Z.PRED_GE, "t0": t, "stream_id": i})
        else:
            qs.append({"kind": Z.PROG_TRIANGLE, "n": n, "seed": seed, "stream_id": i})
            qs.append({"kind": Z.PROG_TRIANGLE, "n": n, "seed": seed + 1, "pred_op": Z.PRED_LT, "t0": t,
                       "stream_id": i})
    return qs


def run_batch(args):
    """One step = one submit of the workload's queries (zg_batch: persistent kernel replayed through
    a CUDA graph).  value: samples/s from CUDA events around the graph launch; e2e: submit + wait
    wall time (descriptors in, counters out)."""
    import numpy as np
    import torch
    import zgraph as Z
    wl = BATCH_WORKLOADS[args.workload]
    Z.init(0)
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    if wl["gen"] == "chung_lu":
        g = Z.Graph.gen_chung_lu(wl["n"], wl["exponent"], wl["avg_degree"], seed=wl["seed"],
                                 max_weight=wl["max_weight"], weight_seed=7)
        qs = batch_queries(Z, np.random.default_rng(3), wl["queries"])
        desc = ("Chung-Lu %d vertices, exponent %.1f, %d edges, edge data in [0, 100); %d queries (%d batch "
                "queries) over triangle / 3-motif / all-predicate / at-least-one-predicate, budgets 2^U(12,24)"
                % (wl["n"], wl["exponent"], g.num_local_edges, wl["queries"], len(qs)))
    else:
        g = Z.Graph.gen_rmat(wl["scale"], wl["edge_factor"], seed=wl["seed"], sampling_only=True)
        star = Z.Program(Z.PROG_PATTERN, pattern=(5, [(0, 1), (0, 2), (0, 3), (0, 4)]))
        house = Z.Program(Z.PROG_PATTERN, pattern=(5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)]))
        n = wl["samples"]
        qs = [{"kind": Z.PROG_FOUR_CLIQUE, "n": n, "seed": 1},
              {"kind": Z.PROG_PATTERN, "program": star, "n": n, "seed": 2},
              {"kind": Z.PROG_PATTERN, "program": house, "n": n, "seed": 3}]
        desc = ("R-MAT scale %d, edge factor %d, %d edges (built on the device); 4-clique, 5-star, 5-house x 2^%d"
                % (wl["scale"], wl["edge_factor"], g.num_local_edges, n.bit_length() - 1))
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    b = Z.Batch(g, max_queries=max(8, len(qs)), cache_bytes=200 << 30)
    t0 = time.perf_counter()
    first = b.run(qs)  # builds the filtered graphs the predicates need
    first_s = time.perf_counter() - t0
    best, ms_variants = b.tune(qs)
    samples = sum(q["n"] for q in qs) + sum(q["n"] for q in qs if q["kind"] == Z.QUERY_THREE_MOTIF)
    for _ in range(max(0, args.warmup - 1)):
        b.run(qs)
    st = torch.cuda.current_stream()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    clocks = ClockSampler(0)
    clocks.start()
    dev_ms, wall = [], []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        b.submit(qs, cuda_stream=st.cuda_stream)
        res = b.wait()
        wall.append(time.perf_counter() - w0)
        dev_ms.append(b.elapsed_ms())  # CUDA events on the stream around the batch's graph launch
    clk = clocks.stop()
    total_ms = sum(dev_ms)
    value = samples * args.steps / (total_ms / 1000.0)
    # algorithmic bytes: access-model sectors per sample of every (program, graph) pair, 2^14 samples
    model_bytes, seen = 0.0, {}
    for q in qs:
        key = (q["kind"], q.get("pred_op", 0), q.get("t0", 0), id(q.get("program")))
        if key not in seen:
            gg = b.filtered_graph(q["pred_op"], q["t0"]) if q.get("pred_op") else g
            if q["kind"] == Z.QUERY_THREE_MOTIF:
                tc, tt = Z.run_three_motif_debug(gg, 1 << 14, 1 << 14, 5)[:2]
                seen[key] = 32.0 * (float(tc["sectors"].mean()) + float(tt["sectors"].mean()))
            else:
                p = q.get("program") or Z.Program(q["kind"])
                seen[key] = 32.0 * float(p.run_debug(gg, 1 << 14, 5)["sectors"].mean())
        model_bytes += seen[key] * q["n"]
    peak, peak_kind = peaks()
    ach = model_bytes / (total_ms / args.steps / 1000.0) / 1e9
    h2d = len(qs) * 72 + 8 * (Z.BATCH_MAX_CHUNKS + max(8, len(qs))) + 16
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int64/u192 exact", "data": "synthetic (device generator)",
            "config": {"workload": "%s: %s" % (args.workload, desc), "queries_per_step": len(qs),
                       "samples_per_step": samples, "graph_gen_and_build_s": round(gen_s, 3),
                       "first_batch_s (builds filtered graphs)": round(first_s, 3),
                       "batch_variant": best, "ms_per_variant": [round(x, 3) for x in ms_variants],
                       "l2": "flushed between steps (512 MiB write)"},
            "e2e": {"value": samples * args.steps / sum(wall), "unit": "samples/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": 2 * 112 * max(8, len(qs)),
                    "queries_per_s": len(qs) * args.steps / sum(wall)},
            "gpu_launches": 3 * args.steps, "clocks": clk,
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "traffic": None, "kernel": "k_batch (all queries of the step)",
                         "peak_source": peak_kind}}
    if wl["gen"] == "rmat":
        line["results"] = {name: {"hits": int(c.hits), "estimate": c.estimate}
                           for name, (c, _) in zip(["four_clique", "five_star", "five_house"], res)}
        if not args.no_time_to_bound:
            line["time_to_bound"] = large_time_to_bound(Z, g)
    elif not args.no_time_to_bound:
        line["learned_batch"] = learned_batch(Z, b, qs)
    print(json.dumps(line), flush=True)


def learned_batch(Z, b, qs, eps=0.05, conf=0.95):
    """The same queries to eps at conf: learned sizing of the whole batch (zg_batch_size_learned:
    pilot batches, one prediction; 3-motif queries keep their budgets), one batch, then top-up
    batches for the answers whose empirical bound does not hold yet (zg_batch_bounded)."""
    model = os.path.join(ROOT, "sampling-graph-mining_gb300", "elp_mlp.npz")
    if not os.path.exists(model):
        return {"skipped": "no trained network at %s" % model}
    net = Z.Mlp.load(model)
    lqs = [q if q["kind"] == Z.QUERY_THREE_MOTIF else {k: v for k, v in q.items() if k != "n"} for q in qs]
    t0 = time.perf_counter()
    sized = b.size_learned(net, lqs, eps, conf)
    sizing_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    total, met, rounds = b.bounded(net, lqs, eps, conf)
    wall = time.perf_counter() - t0
    sized_q = [i for i, q in enumerate(lqs) if q["kind"] != Z.QUERY_THREE_MOTIF]
    return {"eps": eps, "confidence": conf, "queries_sized": len(sized_q), "sizing_s": sizing_s,
            "sized_samples": sum(sized[i]["n"] for i in sized_q),
            "bounded_s": wall, "rounds": rounds, "samples": sum(total[i].samples for i in sized_q),
            "bound_met": sum(1 for i in sized_q if met[i])}


def large_time_to_bound(Z, g, eps=0.01, conf=0.95, cap=1 << 37):
    """Triangle and (unbiased) 4-clique queries to 1 % at 95 % on the largest graph: learned-ELP
    budget, then the empirical-CLT bound check keeps sampling until the bound holds (or the cap)."""
    import elp_learn as EL
    model = os.path.join(ROOT, "sampling-graph-mining_gb300", "elp_mlp.npz")
    if not os.path.exists(model):
        return {"skipped": "no trained network at %s" % model}
    net = Z.Mlp.load(model)
    out = {"eps": eps, "confidence": conf, "max_samples": cap, "patterns": {}}
    for name, kind, exact_kind in (("triangle", Z.PROG_TRIANGLE, Z.EXACT_TRIANGLE),
                                   ("four_clique_unbiased", Z.PROG_FOUR_CLIQUE_UNBIASED, Z.EXACT_FOUR_CLIQUE)):
        prog = Z.Program(kind)
        t0 = time.perf_counter()
        q, n = Z.learned_query(net, g, prog, eps, conf, 77, 4242, stream_id=0x71, max_samples=cap)
        dt = time.perf_counter() - t0
        r = {"n_sized": int(n), "samples": int(q.samples), "bound_met": int(q.bound_met),
             "rel_half_width": q.rel_half_width, "estimate": q.estimate, "seconds": dt}
        if name == "triangle":  # an exact count of the 1.57 G-edge graph's triangles is affordable
            t1 = time.perf_counter()
            ex = g.exact_count(exact_kind)
            r["exact"] = ex
            r["exact_count_seconds"] = time.perf_counter() - t1
            r["rel_err_vs_exact"] = abs(q.estimate - ex) / ex
        out["patterns"][name] = r
    return out


def main():
    args = parse()
    if args.workload in BATCH_WORKLOADS:
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the batched workloads have no CPU arm here: the "
                              "reference runs one query at a time; see the rmat20 workload's reference arm"}))
        else:
            run_batch(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
