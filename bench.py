#!/usr/bin/env python
"""Benchmark of the neighbour-sampling estimator hot path on GB300.

Default workload "rmat26" (the largest single-GPU configuration): undirected R-MAT scale 26, edge
factor 24, a/b/c/d = .57/.19/.19/.05, seed 26, self-loops and duplicates removed (1.57 G edges,
seeded synthetic input generated and built on the device).  One step = the 4-clique, 5-star and
5-house estimators with 2^30 samples each, submitted as one batch (persistent work-queue kernels
replayed through a CUDA graph).

  value : samples/s over the timed steps, device time from CUDA events around the batch's graph
          launch on the launching stream (graph resident in HBM; L2 flushed between steps).
  e2e   : samples/s through the public batch API (zg_batch_submit + zg_batch_wait) with the host
          buffers: every step copies the query descriptors and work list host->device and the
          results device->host (byte counts from zg_batch_copy_bytes); the graph stays resident.
  roofline: bytes the production sampling kernels move per sample (zg_touch_sectors: the same
          kernel with every load's 32-byte sectors counted) x samples / the step's device time,
          against the measured HBM copy peak (the graph is ~300x the L2).
  cpu_baseline: the oracle (CPU restatement of the reference path, all host threads) on the same
          graph, a bounded sample of each program.
  time_to_bound: triangle and unbiased 4-clique queries to 1 % at 95 %, plain ErrorProfile sizing
          vs learned sizing, the same bound check on the same estimators (2 seeds each; the
          triangle's exact count on the device beside it); on R-MAT scale 20 the same comparison
          (3 seeds) and the coverage of 40 independent learned answers of each.

--impl reference times the oracle (the reference's CPU path restated in C, all host threads) on
the same workload and graph, generated on the host by oracle/zgo_gen.c without the GPU library.
Other workloads: rmat20 (R-MAT scale 20, ef 3; four programs x 2^26), rmat13 (scale 13, ef 12;
triangle x 2^20), chunglu_batch (Chung-Lu 4.8 M vertices, 512 mixed predicate queries).
Under torchrun each rank runs its own shard of sample indices (weak scaling, rmat20/rmat13); rank 0
prints one JSON line.
"""
import argparse
import hashlib
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sampling-graph-mining_gb300"))

METRIC = "time-to-1%-error@95% and samples/s, learned vs plain ELP, 1 GB300"
RMAT = {"a": 0.57, "b": 0.19, "c": 0.19}
WORKLOADS = {
    "rmat20": {"gen": "rmat", "scale": 20, "edge_factor": 3, "seed": 1, "samples": 1 << 26,
               "programs": ["triangle", "four_clique", "three_chain", "four_chain"]},
    "rmat13": {"gen": "rmat", "scale": 13, "edge_factor": 12, "seed": 1, "samples": 1 << 20, "programs": ["triangle"]},
    # the Chung-Lu batch's base graph (1.7 GB of device arrays, far above the L2): the four programs
    # alone, for HBM-bound kernel measurements
    "chunglu4": {"gen": "chung_lu", "n": 4800000, "exponent": 2.3, "avg_degree": 18.0, "seed": 2024,
                 "max_weight": 100, "weight_seed": 7, "samples": 1 << 26,
                 "programs": ["triangle", "four_clique", "three_chain", "four_chain"]},
}
BATCH_WORKLOADS = {
    "rmat26": {"gen": "rmat", "scale": 26, "edge_factor": 24, "seed": 26, "samples": 1 << 30,
               "programs": ["four_clique", "five_star", "five_house"]},
    # the headline's programs on R-MAT scale 21 (a few GB on the device): the size an ncu capture of
    # the batch kernels can take, scaled to the headline by samples
    "rmat21_batch": {"gen": "rmat", "scale": 21, "edge_factor": 24, "seed": 26, "samples": 1 << 26,
                     "programs": ["four_clique", "five_star", "five_house"]},
    "chunglu_batch": {"gen": "chung_lu", "n": 4800000, "exponent": 2.3, "avg_degree": 18.0, "seed": 2024,
                      "max_weight": 100, "queries": 512},
}
PROG_IDS = {"triangle": 1, "four_clique": 2, "three_chain": 3, "four_chain": 4, "four_clique_unbiased": 7}
PATTERNS = {"five_star": (5, [(0, 1), (0, 2), (0, 3), (0, 4)]),
            "five_house": (5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)])}
EXACT_IDS = {"triangle": 1, "three_chain": 2, "four_chain": 3, "four_clique": 5, "four_clique_unbiased": 5}
KERNEL_SOURCES = ("zg_internal.cuh", "zg_programs.cuh", "zg_sample_kernel.cuh", "zg_sample.cu", "zg_batch.cu",
                  "zg_graph.cu")
# zg_random_sector_rate's probe kernel and the helpers it uses: its DRAM bytes per sector do not
# depend on the sampling kernels
PROBE_SOURCES = ("zg_internal.cuh", "zg_api.cu")


LAYOUTS = {"auto": 0, "compact": 1, "wide": 2, "packed": 3}
LAYOUT_NAMES = {v: k for k, v in LAYOUTS.items()}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="rmat26", choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-time-to-bound", action="store_true")
    ap.add_argument("--no-coverage", action="store_true")
    ap.add_argument("--l2-fetch", type=int, default=0,
                    help="L2 fetch granularity in bytes for this process (32, 64, 128; 0: the library's)")
    ap.add_argument("--layout", default="auto", choices=sorted(LAYOUTS),
                    help="record layout of the graph (zg_set_record_layout; auto: the library's choice)")
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
        return float(p["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def kernel_source_hash(sources=KERNEL_SOURCES):
    """Hash of the sampling kernels' sources (or of the given csrc files): ties a committed ncu
    traffic figure to the code it was measured on (the GPU host has no git history to compare
    against)."""
    h = hashlib.sha256()
    for name in sources:
        with open(os.path.join(ROOT, "sampling-graph-mining_gb300", "csrc", name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def profile_traffic(kernel, workload, layout):
    """DRAM bytes per sample of `kernel` on `workload` from profiles/dram_traffic.txt (ncu
    dram__bytes_read.sum + dram__bytes_write.sum per launch / samples per launch), used only when the
    record layout and the kernel-source hash it was captured at match this build; else None with
    the reason."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        lines = [l.split() for l in open(path) if l.strip() and not l.startswith("#")]
    except OSError:
        return None, "no capture committed"
    cur = kernel_source_hash()
    for f in lines:
        if len(f) >= 6 and f[0] == kernel and f[1] == workload:
            if f[2] != layout:
                return None, "capture taken with %s records, this graph has %s" % (f[2], layout)
            if f[3] != cur:
                return None, "stale: captured at kernel-source hash %s, this build is %s" % (f[3], cur)
            return float(f[4]) / float(f[5]), "ncu capture (%s)" % " ".join(f[6:]) if len(f) > 6 else "ncu capture"
    return None, "no capture of %s on %s" % (kernel, workload)


def workload_config(name, m):
    """The workload as both arms print it (same dict, so the two lines compare like for like)."""
    wl = BATCH_WORKLOADS.get(name) or WORKLOADS[name]
    if wl["gen"] == "rmat":
        graph = "R-MAT scale %d, edge factor %d, a/b/c/d=.57/.19/.19/.05, seed %d" % (wl["scale"], wl["edge_factor"],
                                                                                   wl["seed"])
    else:
        graph = "Chung-Lu %d vertices, exponent %.1f, average degree %.0f, seed %d" % (wl["n"], wl["exponent"],
                                                                                     wl["avg_degree"], wl["seed"])
    desc = ("%s: %s, simplified (%d undirected edges); one step = %s estimators x 2^%d samples each"
            % (name, graph, m, " + ".join(wl["programs"]), wl["samples"].bit_length() - 1))
    return {"workload": desc, "inputs": "graph built before the timed steps and kept resident (GPU arm: device memory, L2 flushed "
                                           "between steps)"}


# ---- CPU side (oracle): cpu_baseline and the reference arm -------------------------------------
def oracle_programs(O, names):
    out = []
    for name in names:
        if name in PATTERNS:
            nv, pe = PATTERNS[name]
            out.append((name, O.OracleProgram(6, pattern=(nv, pe)), 6))
        else:
            out.append((name, O.OracleProgram(PROG_IDS[name]), PROG_IDS[name]))
    return out


def oracle_rates(O, og, names, threads, target_s):
    """Samples/s of each program on the oracle graph: n doubles until one run takes target_s / 4."""
    rates, total_n, total_s = {}, 0, 0.0
    budget = target_s / len(names)
    for name, prog, kind in oracle_programs(O, names):
        n = 1 << 10
        while True:
            t0 = time.perf_counter()
            O.run(og, prog, n, 0, 17, kind, threads)
            dt = time.perf_counter() - t0
            if dt > budget / 4 or n >= (1 << 28):
                break
            n *= 4
        rates[name] = n / dt
        total_n += n
        total_s += dt
    return rates, total_n, total_s


def cpu_baseline(edges, nv, names, threads, target_s=16.0, with_time_to_bound=True):
    """The oracle (CPU restatement of the reference path) on a bounded sample of the workload, and
    (with_time_to_bound) the reference's own host time to a 1 %/95 % triangle answer on the graph."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    t0 = time.perf_counter()
    og = O.OracleGraph(edges, nv)
    build_s = time.perf_counter() - t0
    rates, total_n, total_s = oracle_rates(O, og, names, threads, target_s)
    out = {"value": total_n / total_s, "unit": "samples/s", "cores": threads, "kind": "port",
           "sample": "%s: %d samples in total (the last, longest run per program), oracle/zg_oracle.c with %d threads "
                     "on the same graph (oracle graph build %.1f s); per program %s"
                     % (",".join(names), total_n, threads, build_s, {k: round(v) for k, v in rates.items()})}
    if with_time_to_bound:
        try:
            out["time_to_bound"] = cpu_time_to_bound(O, edges, nv, og, threads)
        except Exception as exc:  # the samples/s figure stands on its own
            out["time_to_bound"] = {"error": "%s: %s" % (type(exc).__name__, exc)}
    return out


def run_reference(args):
    """The reference arm: the oracle (the reference's CPU path restated in C) with all host threads
    on the same graph, generated on the host (oracle/zgo_gen.c, edge for edge the device generator's
    graph) without the GPU library; each step a bounded sample of every program."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    wl = BATCH_WORKLOADS.get(args.workload) or WORKLOADS[args.workload]
    if wl["gen"] != "rmat":
        print(json.dumps({"impl": "reference", "unavailable": "the Chung-Lu workloads have no CPU arm (the oracle's "
                          "host generator is R-MAT's); see the rmat26 and rmat20 workloads' reference arms"}), flush=True)
        return
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    edges = O.gen_rmat(wl["scale"], wl["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"], wl["seed"])
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    og = O.OracleGraph(edges, 1 << wl["scale"])
    build_s = time.perf_counter() - t0
    progs = oracle_programs(O, wl["programs"])
    # a bounded per-step sample: about one second of CPU per step
    n = 1 << 8
    while True:
        t0 = time.perf_counter()
        for _, p, kind in progs:
            O.run(og, p, n, 0, 5, kind, threads)
        dt = time.perf_counter() - t0
        if dt > 0.5 or n >= wl["samples"]:
            break
        n *= 2
    for i in range(args.warmup):
        for j, (_, p, kind) in enumerate(progs):
            O.run(og, p, n, i * n, 5 + j, kind, threads)
    per_prog = [0.0] * len(progs)
    t0 = time.perf_counter()
    for i in range(args.steps):
        for j, (_, p, kind) in enumerate(progs):
            t1 = time.perf_counter()
            O.run(og, p, n, (args.warmup + i) * n, 5 + j, kind, threads)
            per_prog[j] += time.perf_counter() - t1
    dt = time.perf_counter() - t0
    value = len(progs) * n * args.steps / dt
    sample = ("%d samples of each of %d programs per step (bounded sample of the 2^%d per program), "
              "oracle/zg_oracle.c on %d host threads; graph generated on the host in %.1f s, oracle graph built in %.1f s"
              % (n, len(progs), wl["samples"].bit_length() - 1, threads, gen_s, build_s))
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1000 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int64/f64", "data": "synthetic (seeded R-MAT)",
            "impl": "reference", "config": workload_config(args.workload, len(edges)),
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    # each program's share of the timed steps, and its closure checks (conditional_close look-ups up
    # to the first missing edge, the access model's count, from the traces of 2^14 samples)
    line["per_program"] = []
    for j, (name, p, kind) in enumerate(progs):
        closures = float(O.traces(og, p, 1 << 14, 5 + j, stream=kind, threads=threads)[0]["closures"].mean())
        rate = n * args.steps / per_prog[j]
        line["per_program"].append({"program": name, "samples_per_s": rate, "closure_checks_per_sample": closures,
                                    "closure_checks_per_s": closures * rate})
    if not args.no_time_to_bound:
        try:
            line["time_to_bound"] = cpu_time_to_bound(O, edges, 1 << wl["scale"], og, threads)
        except Exception as exc:  # the samples/s line above stands on its own
            line["time_to_bound"] = {"error": "%s: %s" % (type(exc).__name__, exc)}
    print(json.dumps(line), flush=True)


def cpu_time_to_bound(O, edges, nv, og, threads, seed=31, eps=0.01, conf=0.95, min_run_s=2.0):
    """The reference's own way to a 1 %/95 % triangle answer on the host: ErrorProfile::run, i.e.
    get_num_estimators (timed: the host restatement with zg_elp_plain's draw plan, so n_required is
    the count the GPU arm's plain sizing gets for the same seed) followed by calculate(n_required)
    (its time from the measured samples/s of the triangle program on the whole graph; the billions
    of samples are not run)."""
    prog = O.OracleProgram(PROG_IDS["triangle"])
    t0 = time.perf_counter()
    n_req = O.plain_elp(edges, nv, prog, 1, seed, eps, conf, og.m, og.max_degree, threads)
    profile_s = time.perf_counter() - t0
    n = 1 << 14
    while True:
        t0 = time.perf_counter()
        O.run(og, prog, n, seed + 100, 0x51, 0, threads)
        dt = time.perf_counter() - t0
        if dt >= min_run_s or n >= 1 << 36:
            break
        n *= 2
    rate = n / dt
    return {"pattern": "triangle", "eps": eps, "confidence": conf, "elp_seed": seed, "n_required": n_req,
            "profile_s": profile_s, "samples_per_s": rate, "calculate_s": n_req / rate,
            "seconds": profile_s + n_req / rate, "cores": threads,
            "method": "ErrorProfile::get_num_estimators on the host (oracle.plain_elp: 10 %% subsample, 2^14 x 16 + "
                      "2^23 estimators, regression), timed; then calculate(n_required) at the triangle's measured "
                      "samples/s (%d samples in %.2f s), not run" % (n, dt)}


# ---- GPU side ---------------------------------------------------------------------------------
def make_program(Z, name):
    if name in PATTERNS:
        return Z.Program(Z.PROG_PATTERN, pattern=PATTERNS[name])
    return Z.Program(PROG_IDS[name])


def touch_bytes(Z, g, progs, names, seed, n=1 << 20):
    """Bytes per sample each production sampling kernel moves (zg_touch_sectors on n samples)."""
    return {name: p.touch_bytes_per_sample(g, n, seed) for name, p in zip(names, progs)}


def time_to_bound(Z, g, names, exact, eps=0.01, conf=0.95, cap=1 << 37, seed=31, repeats=1):
    """Time from query submission (graph resident) to an answer whose 95 % half-width is <= 1 % of
    the estimate: plain ErrorProfile sizing vs the learned network, the same bound check, the same
    estimators (common random numbers), `repeats` independent seeds per pattern (the speed-up is
    the ratio of the mean times).  4-cliques run the unbiased canonical-path program: the
    reference's estimator finds ~60 % of the cliques, so a tight interval around it is not an
    accuracy claim."""
    import elp_learn as EL
    model = os.path.join(ROOT, "sampling-graph-mining_gb300", "elp_mlp.npz")
    if not os.path.exists(model):
        return {"skipped": "no trained network at %s" % model}
    net = Z.Mlp.load(model)
    out = {"eps": eps, "confidence": conf, "max_samples": cap, "model": "sampling-graph-mining_gb300/elp_mlp.npz",
           "patterns": {}}
    for name in names:
        runs = [EL.compare(net, g, name, eps=eps, conf=conf, seed=seed + 1000 * i, max_samples=cap)
                for i in range(repeats)]
        ex = exact.get(name)
        for r in runs:
            for k in ("plain", "learned"):
                r[k]["rel_err_vs_exact"] = abs(r[k]["estimate"] - ex) / ex if ex else None
        r = dict(runs[0]) if repeats == 1 else {"pattern": name, "runs": runs}
        for k in ("plain", "learned"):
            r["mean_seconds_" + k] = sum(x[k]["seconds"] for x in runs) / repeats
            r["mean_samples_" + k] = sum(x[k]["samples"] for x in runs) / repeats
        r["exact"] = ex
        r["speedup_learned_over_plain"] = r["mean_seconds_plain"] / r["mean_seconds_learned"]
        out["patterns"][name] = r
    return out


def random_sector_bytes():
    """DRAM bytes one random 32-byte sector read moves: the ncu capture of zg_random_sector_rate's
    kernel in profiles/dram_traffic.txt (bytes of the timed launch / its sectors), used while the
    probe's own sources (PROBE_SOURCES) hash to the value it was captured at."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        lines = [l.split() for l in open(path) if l.strip() and not l.startswith("#")]
    except OSError:
        return None, "no capture committed"
    for f in lines:
        if len(f) >= 6 and f[0] == "k_random_sectors":
            if f[3] != kernel_source_hash(PROBE_SOURCES):
                return None, "stale: captured at probe-source hash %s" % f[3]
            return float(f[4]) / float(f[5]), "ncu capture on %s" % f[1]
    return None, "no capture of k_random_sectors"


def random_sector_view(Z, g, touched_gbs, dram_gbs=None, near_l2=False):
    """The sampling loads are isolated 32-byte sectors at random addresses: their ceiling is the rate
    at which the memory system serves such reads, measured live after the timed steps by
    zg_random_sector_rate over this graph's records and adjacency.  `frac` compares the sectors the
    kernels touch (some share a line, so it can exceed 1); `dram` compares the DRAM bytes the
    kernels move (ncu) with the DRAM bytes the probe moves at its rate."""
    peak = Z.random_sector_rate(g, 256)
    ach = touched_gbs * 1e9 / 32.0
    out = {"achieved": ach / 1e9, "peak": peak / 1e9, "unit": "G sectors/s", "frac": ach / peak if peak else None,
           "peak_source": "measured live: zg_random_sector_rate (8 independent 32-byte loads in flight per thread, "
                          "one full-occupancy grid, over this graph's records and edge-id-ordered adjacency)"}
    bps, src = random_sector_bytes()
    if near_l2:
        out["dram"] = None
        out["dram_source"] = "near-L2 graph: the probe's sectors mostly hit L2, its DRAM bytes per sector do not apply"
    elif dram_gbs and bps and peak:
        ceiling = peak * bps / 1e9
        out["dram"] = {"achieved_gbs": dram_gbs, "ceiling_gbs": ceiling, "frac": dram_gbs / ceiling,
                       "bytes_per_random_sector": bps, "source": src}
    else:
        out["dram"] = None
        out["dram_source"] = src if not bps else "no DRAM capture of the kernels at this build"
    return out


def wilson(k, n, z=1.959963984540054):
    """Wilson score 95 % interval of a binomial fraction k/n."""
    if n == 0:
        return [0.0, 1.0]
    p = k / n
    c = (p + z * z / (2 * n)) / (1 + z * z / n)
    h = z * math.sqrt(p * (1 - p) / n + z * z / (4 * n * n)) / (1 + z * z / n)
    return [round(c - h, 4), round(c + h, 4)]


def coverage(Z, g, exact, queries, eps=0.01, conf=0.95, cap=1 << 37):
    """Delivered accuracy: independent queries (learned sizing + bound check; seeds 1000 + s), how
    many met their bound, how many intervals hold the exact count, and how many answers landed
    within eps of it, with the Wilson 95 % interval of the covered fraction."""
    model = os.path.join(ROOT, "sampling-graph-mining_gb300", "elp_mlp.npz")
    if not os.path.exists(model):
        return {"skipped": "no trained network at %s" % model}
    net = Z.Mlp.load(model)
    out = {}
    for name, nq in queries.items():
        prog = Z.Program(PROG_IDS[name])
        ex = exact[name]
        inside, covered, met, samples, t0 = 0, 0, 0, 0, time.perf_counter()
        for s in range(nq):
            q = Z.learned_query(net, g, prog, eps, conf, 1000 + s, 5000 + s, stream_id=0x60 + s, max_samples=cap)[0]
            met += q.bound_met
            inside += abs(q.estimate - ex) <= eps * ex
            covered += abs(q.estimate - ex) <= q.half_width
            samples += q.samples
        out[name] = {"queries": nq, "eps": eps, "bound_met": met, "interval_holds_exact": covered,
                     "covered_fraction_wilson95": wilson(covered, nq), "within_eps_of_exact": inside, "exact": ex,
                     "mean_samples": samples / nq, "seconds": time.perf_counter() - t0}
    return out


def run_gb300(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import zgraph as Z
    Z.init(local)
    l2_fetch = Z.set_l2_fetch_granularity(args.l2_fetch)
    Z.set_record_layout(LAYOUTS[args.layout])
    wl = WORKLOADS[args.workload]
    n = wl["samples"]
    t0 = time.perf_counter()
    if wl["gen"] == "rmat":
        nv = 1 << wl["scale"]
        g = Z.Graph.gen_rmat(wl["scale"], wl["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"], wl["seed"])
    else:
        nv = wl["n"]
        g = Z.Graph.gen_chung_lu(wl["n"], wl["exponent"], wl["avg_degree"], seed=wl["seed"],
                                 max_weight=wl["max_weight"], weight_seed=wl["weight_seed"])
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    names = wl["programs"]
    progs = [make_program(Z, p) for p in names]
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    tuning = {}
    fixed = dict(kv.split("=") for kv in args.variants.split(",")) if args.variants else None
    for name, p in zip(names, progs):
        if fixed is not None:
            if name in fixed:
                p.set_variant(int(fixed[name]))
            tuning[name] = dict(p.variant(), fixed=True)
            continue
        # probes of 2^23 samples; 2^26 on wide-record graphs, whose grids hold six times the
        # resident blocks (a probe must give every thread more than a few samples)
        probe_log2 = 26 if g.meta().record_layout == Z.RECORDS_WIDE else 23
        best, ms = p.tune(g, 1 << probe_log2, cuda_stream=sp)
        tuning[name] = {"variant": best, "min_blocks": p.variant()["min_blocks"],
                        "ms_per_variant_2^%d" % probe_log2: [round(x, 3) for x in ms]}
    d_res = torch.zeros((len(progs), Z.RESULT_BYTES), dtype=torch.uint8, device="cuda")
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

    # end to end through the public API: calculate() per program, each result read back
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
           "d2h_bytes_per_step": len(insts) * Z.RESULT_BYTES,
           "note": "calculate() per program; the graph is resident and a query's inputs are scalars (no host "
                   "buffer to copy in); each result (112 bytes) is read back"}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    touched = touch_bytes(Z, g, progs, names, seed)
    closures = {name: float(p.run_debug(g, 1 << 16, seed, stream_id=j + 1)["closures"].mean())
                for j, (name, p) in enumerate(zip(names, progs))}
    hbm, hbm_src = peaks()
    l2_gbs = Z.read_bandwidth(48 << 20, 100)
    layout = LAYOUT_NAMES[g.meta().record_layout]
    kern = []
    for j, name in enumerate(names):
        t = per_prog[j] / args.steps / 1000.0
        dram_ps, dram_src = profile_traffic("k_sample<%s>" % name, args.workload, layout)
        kern.append({"kernel": "k_sample<%s>" % name, "ms": per_prog[j] / args.steps, "samples_per_s": n / t,
                     "touched_bytes_per_sample": touched[name], "touched_gbs": touched[name] * n / t / 1e9,
                     "dram_bytes_per_sample": dram_ps, "dram_source": dram_src,
                     "dram_gbs": dram_ps * n / t / 1e9 if dram_ps else None,
                     "closure_checks_per_sample": closures[name], "closure_checks_per_s": closures[name] * n / t,
                     "hits": int(res[j].hits), "estimate": res[j].estimate})
    dom = max(kern, key=lambda k: k["ms"])
    # A graph whose sampling working set is about the L2 size (R-MAT scale 20) is bound by the L2
    # read bandwidth (measured live); a larger one by HBM.  The DRAM figure says how much came from HBM.
    near_l2 = g.meta().device_bytes < (1 << 30)
    bpeak = l2_gbs if near_l2 else hbm
    roofline = {"bound": "l2" if near_l2 else "hbm", "achieved": dom["touched_gbs"], "peak": bpeak, "unit": "GB/s",
                "frac": dom["touched_gbs"] / bpeak, "kernel": dom["kernel"],
                "traffic": dom["dram_bytes_per_sample"] * n if dom["dram_bytes_per_sample"] else None,
                "traffic_source": dom["dram_source"],
                "algorithmic_bytes": "zg_touch_sectors: 32-byte sectors the kernel's loads touch, per sample x samples",
                "peak_source": ("measured live: reads of a 48 MiB buffer resident in L2 (zg_read_bandwidth)" if near_l2
                                else hbm_src),
                "l2": {"peak": l2_gbs, "frac": dom["touched_gbs"] / l2_gbs},
                "hbm": {"peak": hbm, "peak_source": hbm_src,
                        "dram_frac": dom["dram_gbs"] / hbm if dom["dram_gbs"] else None},
                "random_sectors": random_sector_view(Z, g, dom["touched_gbs"], dom["dram_gbs"], near_l2),
                "per_kernel": kern}
    exact, acc = {}, {}
    ttb = None
    if not args.no_time_to_bound:
        for j, name in enumerate(names):
            ex = g.exact_count(EXACT_IDS[name])
            exact[name] = ex
            acc[name] = {"exact": ex, "estimate": res[j].estimate,
                         "rel_err": abs(res[j].estimate - ex) / ex if ex else None}
        if "four_clique" in names:
            exact["four_clique_unbiased"] = exact["four_clique"]
        ttb = time_to_bound(Z, g, [x for x in ("triangle", "four_clique_unbiased") if x in exact], exact)
        if not args.no_coverage:
            ttb["coverage"] = coverage(Z, g, exact, {x: 400 if x == "triangle" else 40
                                                     for x in ("triangle", "four_clique_unbiased") if x in exact})
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int64/u192 exact (f64 reference 1/p)",
            "data": "synthetic (seeded R-MAT, generated on the device)",
            "config": workload_config(args.workload, g.num_local_edges),
            "setup": {"graph_gen_and_build_s": round(build_s, 3), "graph_device_bytes": int(g.meta().device_bytes),
                      "record_layout": layout, "launch_tuning": tuning,
                      "l2_fetch_bytes": args.l2_fetch or l2_fetch},
            "e2e": e2e, "gpu_launches": 2 * len(progs) * args.steps, "clocks": clk, "roofline": roofline,
            "accuracy": acc, "time_to_bound": ttb}
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(g.download_edges(), nv, names, os.cpu_count() or 1)
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
    """One step = one submit of the workload's queries (zg_batch: persistent kernels replayed through
    a CUDA graph).  value: samples/s from CUDA events around the graph launch; e2e: submit + wait
    wall time (descriptors in, counters out)."""
    import numpy as np
    import torch
    import zgraph as Z
    wl = BATCH_WORKLOADS[args.workload]
    Z.init(0)
    torch.cuda.set_device(0)
    l2_fetch = Z.set_l2_fetch_granularity(args.l2_fetch)
    Z.set_record_layout(LAYOUTS[args.layout])
    t0 = time.perf_counter()
    rmat = wl["gen"] == "rmat"
    if not rmat:
        g = Z.Graph.gen_chung_lu(wl["n"], wl["exponent"], wl["avg_degree"], seed=wl["seed"],
                                 max_weight=wl["max_weight"], weight_seed=7)
        qs = batch_queries(Z, np.random.default_rng(3), wl["queries"])
        nv = wl["n"]
        config = {"workload": "%s: Chung-Lu %d vertices, exponent %.1f, %d edges, edge data in [0, 100); %d queries (%d "
                              "batch queries) over triangle / 3-motif / all-predicate / at-least-one-predicate, budgets "
                              "2^U(12,24)" % (args.workload, wl["n"], wl["exponent"], g.num_local_edges, wl["queries"],
                                              len(qs)),
                  "inputs": "graph built before the timed steps and kept resident (GPU arm: device memory, L2 flushed "
                                           "between steps)"}
        names = []
    else:
        g = Z.Graph.gen_rmat(wl["scale"], wl["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"], seed=wl["seed"],
                             sampling_only=True)
        nv = 1 << wl["scale"]
        names = wl["programs"]
        progs = {name: make_program(Z, name) for name in names}
        qs = []
        for j, name in enumerate(names):
            q = {"kind": progs[name].kind, "n": wl["samples"], "seed": j + 1}
            if name in PATTERNS:
                q["program"] = progs[name]
            qs.append(q)
        config = workload_config(args.workload, g.num_local_edges)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    b = Z.Batch(g, max_queries=max(8, len(qs)), cache_bytes=200 << 30)
    t0 = time.perf_counter()
    b.run(qs)  # builds the filtered graphs the predicates need
    first_s = time.perf_counter() - t0
    best, ms_variants = b.tune(qs)
    samples = sum(q["n"] for q in qs) + sum(q["n"] for q in qs if q["kind"] == Z.QUERY_THREE_MOTIF)
    for _ in range(max(0, args.warmup - 1)):
        b.run(qs)
    st = torch.cuda.current_stream()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    h2d, d2h = b.copy_bytes()
    clocks = ClockSampler(0)
    clocks.start()
    dev_ms, wall = [], []
    res = None
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
    hbm, hbm_src = peaks()
    layout = LAYOUT_NAMES[g.meta().record_layout]
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int64/u192 exact", "data": "synthetic (device generator)",
            "config": config,
            "setup": {"graph_gen_and_build_s": round(gen_s, 3), "graph_device_bytes": int(g.meta().device_bytes),
                      "record_layout": layout, "queries_per_step": len(qs), "samples_per_step": samples,
                      "first_batch_s": round(first_s, 3), "batch_variant": best, "l2_fetch_bytes": args.l2_fetch or l2_fetch,
                      "ms_per_variant": [round(x, 3) for x in ms_variants]},
            "e2e": {"value": samples * args.steps / sum(wall), "unit": "samples/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "queries_per_s": len(qs) * args.steps / sum(wall),
                    "note": "zg_batch_submit + zg_batch_wait from host buffers: query descriptors and work list in, "
                            "results out; the graph stays resident"},
            "gpu_launches": 3 * args.steps, "clocks": clk}
    if rmat:
        # bytes the production kernels move per sample, and each program alone (CUDA events, k_sample)
        touched = touch_bytes(Z, g, [progs[x] for x in names], names, 1)
        step_bytes = sum(touched[x] * wl["samples"] for x in names)
        achieved = step_bytes / (total_ms / args.steps / 1000.0) / 1e9
        stream = torch.cuda.current_stream()
        d_res = torch.zeros(Z.RESULT_BYTES, dtype=torch.uint8, device="cuda")
        # conditional_close look-ups per sample (the access model's count, up to the first missing
        # edge) from the debug kernel's traces: the 4-clique closes three edges; the generic pattern
        # programs sample every edge and close none
        closures = {name: float(progs[name].run_debug(g, 1 << 16, j + 1)["closures"].mean())
                    for j, name in enumerate(names)}
        kern = []
        for j, name in enumerate(names):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            # one untimed launch first (the program's first launch sets up its launch shape)
            progs[name].run_async(g, 1 << 20, j + 1, d_res.data_ptr(), cuda_stream=stream.cuda_stream)
            flush.zero_()
            e0.record(stream)
            progs[name].run_async(g, wl["samples"], j + 1, d_res.data_ptr(), cuda_stream=stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            dram_ps, dram_src = profile_traffic("k_sample<%s>" % name, args.workload, layout)
            kern.append({"kernel": "k_sample<%s> (the program alone)" % name, "ms": ms,
                         "samples_per_s": wl["samples"] / (ms / 1000.0), "touched_bytes_per_sample": touched[name],
                         "touched_gbs": touched[name] * wl["samples"] / (ms / 1000.0) / 1e9,
                         "frac_of_hbm_peak": touched[name] * wl["samples"] / (ms / 1000.0) / 1e9 / hbm,
                         "closure_checks_per_sample": closures[name],
                         "closure_checks_per_s": closures[name] * wl["samples"] / (ms / 1000.0),
                         "dram_bytes_per_sample": dram_ps, "dram_source": dram_src})
        dram_ps, dram_src = profile_traffic("k_batch", args.workload, layout)
        line["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                            "kernel": "k_batch + k_batch_pattern (the step's sampling kernels, one CUDA graph)",
                            "traffic": dram_ps * samples if dram_ps else None, "traffic_source": dram_src,
                            "algorithmic_bytes": "zg_touch_sectors: 32-byte sectors the production kernels' loads "
                                                 "touch per sample (%s) x 2^30 samples per program"
                                                 % {k: round(v, 1) for k, v in touched.items()},
                            "dram": ({"gbs": dram_ps * samples / (total_ms / args.steps / 1000.0) / 1e9,
                                      "frac": dram_ps * samples / (total_ms / args.steps / 1000.0) / 1e9 / hbm,
                                      "note": "DRAM bytes with the default 128-byte L2 fills; the kernels are bound "
                                              "by load latency (the same time with 32-byte fills at the touched "
                                              "bytes)"} if dram_ps else None),
                            "bound_note": "latency of each sample's dependent loads (profiles/k_batch_pattern_rmat21.md)",
                            "random_sectors": random_sector_view(
                                Z, g, achieved,
                                dram_ps * samples / (total_ms / args.steps / 1000.0) / 1e9 if dram_ps else None),
                            "peak_source": hbm_src, "per_kernel": kern}
        line["results"] = {name: {"hits": int(c.hits), "estimate": c.estimate} for name, (c, _) in zip(names, res)}
        if not args.no_time_to_bound:
            t1 = time.perf_counter()
            exact = {"triangle": g.exact_count(EXACT_IDS["triangle"]), "four_clique_unbiased": None}
            exact_s = time.perf_counter() - t1
            line["time_to_bound"] = time_to_bound(Z, g, ["triangle", "four_clique_unbiased"], exact, repeats=2)
            line["time_to_bound"]["exact_triangle_count"] = {"value": exact["triangle"], "seconds": exact_s,
                                                            "kernel": "zg_exact_count (degree-oriented DAG)"}
            if not args.no_coverage:
                line["time_to_bound"]["rmat20"] = rmat20_bounds(Z)
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(g.download_edges(), nv, names, os.cpu_count() or 1)
    else:
        # algorithmic bytes: the sectors every (program, graph) pair's production kernel touches
        bytes_step, seen = 0.0, {}
        for q in qs:
            key = (q["kind"], q.get("pred_op", 0), q.get("t0", 0))
            if key not in seen:
                gg = b.filtered_graph(q["pred_op"], q["t0"]) if q.get("pred_op") else g
                if q["kind"] == Z.QUERY_THREE_MOTIF:
                    seen[key] = sum(Z.Program(k).touch_bytes_per_sample(gg, 1 << 16, 5) for k in (3, 1))
                else:
                    seen[key] = Z.Program(q["kind"]).touch_bytes_per_sample(gg, 1 << 16, 5)
            bytes_step += seen[key] * q["n"]
        ach = bytes_step / (total_ms / args.steps / 1000.0) / 1e9
        dram_ps, dram_src = profile_traffic("k_batch", args.workload, layout)
        line["roofline"] = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                            "kernel": "k_batch (all queries of the step)",
                            "traffic": dram_ps * samples if dram_ps else None, "traffic_source": dram_src,
                            "algorithmic_bytes": "zg_touch_sectors of each (program, graph) pair x its samples",
                            "random_sectors": random_sector_view(Z, g, ach),
                            "peak_source": hbm_src}
        if not args.no_time_to_bound:
            line["learned_batch"] = learned_batch(Z, b, qs)
    print(json.dumps(line), flush=True)


def rmat20_bounds(Z):
    """On R-MAT scale 20 (whose exact counts are cheap): plain vs learned time to the 1 %/95 % bound
    for the triangle and the unbiased 4-clique (3 seeds each), and the coverage of independent
    learned answers (400 triangle and 40 unbiased 4-clique answers at 1 %; 400 unbiased 4-clique
    answers at 5 % on R-MAT scale 16)."""
    wl = WORKLOADS["rmat20"]
    g = Z.Graph.gen_rmat(wl["scale"], wl["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"], wl["seed"],
                         sampling_only=False)
    exact = {"triangle": g.exact_count(EXACT_IDS["triangle"]),
             "four_clique_unbiased": g.exact_count(EXACT_IDS["four_clique"])}
    out = {"graph": "rmat20: R-MAT scale 20, edge factor 3, seed 1 (%d edges)" % g.num_local_edges}
    out["time_to_bound"] = time_to_bound(Z, g, ["triangle", "four_clique_unbiased"], exact, repeats=3)
    # 400 triangle answers (each a few ms) and 40 unbiased 4-clique answers (each ~2 s) at 1 %
    out["coverage"] = coverage(Z, g, exact, {"triangle": 400, "four_clique_unbiased": 40})
    # more 4-clique answers at 5 % on R-MAT scale 16, edge factor 16 (each a few ms)
    g16 = Z.Graph.gen_rmat(16, 16, RMAT["a"], RMAT["b"], RMAT["c"], 1, sampling_only=False)
    ex16 = {"four_clique_unbiased": g16.exact_count(EXACT_IDS["four_clique"])}
    out["coverage_rmat16_5pct"] = coverage(Z, g16, ex16, {"four_clique_unbiased": 400}, eps=0.05)
    return out


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


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload in BATCH_WORKLOADS:
        run_batch(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
