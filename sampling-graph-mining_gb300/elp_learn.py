"""Learned error-latency profile: training data from the plain estimator, training of the
network by the library's own CUDA kernels, and budget sizing.

The network (zg_mlp_*) maps 16 query features (zg_graph_features: degree statistics of the
graph, the pattern class, an adaptive pilot of 2^16..2^22 estimators) to log2 of the per-sample relative variance
Var(1/p) / E(1/p)^2 and log2 of the per-sample latency.  For a target error eps at confidence
conf the budget is n = z^2 * cv2 / eps^2; zg_query then checks the answer against its empirical
bound and keeps sampling if needed, so a wrong prediction costs time, never accuracy.

Training rows come from the plain estimator on seeded synthetic graphs: R-MAT with a in
[0.45, 0.65] (b = c = (1 - a - 0.05) / 2) and Chung-Lu with exponent in [2.1, 3.0]; the target
variance is measured on long runs (at least min_hits hits), the latency by wall time.

  python sampling-graph-mining_gb300/elp_learn.py --graphs 256 --heldout 32 --out elp_mlp.npz
"""
import argparse
import json
import math
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import zgraph as Z  # noqa: E402

STAR = (5, [(0, 1), (0, 2), (0, 3), (0, 4)])
HOUSE = (5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)])
PATTERNS = {
    "triangle": (Z.PROG_TRIANGLE, 0, None),
    "four_clique": (Z.PROG_FOUR_CLIQUE, 0, None),
    "three_chain": (Z.PROG_THREE_CHAIN, 0, None),
    "four_chain": (Z.PROG_FOUR_CHAIN, 0, None),
    "star5": (Z.PROG_PATTERN, 0, STAR),
    "house5": (Z.PROG_PATTERN, 0, HOUSE),
    "four_clique_unbiased": (Z.PROG_FOUR_CLIQUE_UNBIASED, 0, None),
}


def graph_specs(count, seed, min_scale=12, max_scale=20, edge_factor=(4, 16)):
    """Seeded mix of R-MAT and Chung-Lu graph descriptions."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        scale = int(rng.integers(min_scale, max_scale + 1))
        if i % 2 == 0:
            a = float(rng.uniform(0.45, 0.65))
            bc = (1.0 - a - 0.05) / 2.0
            out.append({"kind": "rmat", "scale": scale, "edge_factor": int(rng.integers(*edge_factor)), "a": a,
                        "b": bc, "c": bc, "seed": int(rng.integers(1, 1 << 30))})
        else:
            out.append({"kind": "chung_lu", "n": 1 << scale, "exponent": float(rng.uniform(2.1, 3.0)),
                        "avg_degree": float(rng.uniform(*edge_factor)) * 2.0, "seed": int(rng.integers(1, 1 << 30))})
    return out


def build_graph(spec):
    """The spec's graph, generated and built on the device (equal to the host generators' output)."""
    if spec["kind"] == "rmat":
        return Z.Graph.gen_rmat(spec["scale"], spec["edge_factor"], spec["a"], spec["b"], spec["c"], spec["seed"],
                                sampling_only=True)
    return Z.Graph.gen_chung_lu(spec["n"], spec["exponent"], spec["avg_degree"], spec["seed"], sampling_only=True)


def measure(graph, program, seed, min_hits=200, start=1 << 20, max_samples=1 << 30):
    """Per-sample relative variance and latency of the plain estimator (long runs)."""
    n, first, hits, sw2 = start, 0, 0, 0.0
    total = None
    t_run, n_run = 0.0, 0
    while True:
        t0 = time.perf_counter()
        c = program.run(graph, n, seed, stream_id=0x4C45, first_sample=first)
        dt = time.perf_counter() - t0
        t_run += dt
        n_run += n
        s = c.exact_sum()
        total = s if total is None else total + s
        hits += c.hits
        sw2 += c.sum_w2
        first += n
        if hits >= min_hits or first >= max_samples:
            break
        n = min(n * 4, max_samples - first)
    if hits < 2:
        return None
    mean = float(total / first)
    cv2 = (sw2 / first) / (mean * mean) - 1.0
    return {"cv2": cv2, "ns_per_sample": 1e9 * t_run / n_run, "mean": mean, "samples": first, "hits": hits}


def make_dataset(specs, patterns=PATTERNS, seed=11, log=None):
    X, Y, meta = [], [], []
    for gi, spec in enumerate(specs):
        g = build_graph(spec)
        for name, (kind, param, pat) in patterns.items():
            prog = Z.Program(kind, param, pat)
            f = Z.features(g, prog, 0, seed + gi)  # adaptive pilot, as zg_elp_learned uses
            mres = measure(g, prog, seed + gi)
            if mres is None or not (mres["cv2"] > 0):
                continue
            X.append(f)
            Y.append([math.log2(mres["cv2"]), math.log2(mres["ns_per_sample"])])
            meta.append({"graph": gi, "pattern": name, **mres})
        g.free()
        if log:
            log("graph %d/%d done (%d rows)" % (gi + 1, len(specs), len(X)))
    return np.array(X, np.float32), np.array(Y, np.float32), meta


def train(X, Y, seed=3, epochs=400, batch=32, lr=2e-3):
    net = Z.Mlp(seed)
    loss = net.train(X, Y, epochs=epochs, batch=min(batch, 64), lr=lr, seed=seed)
    return net, loss


def compare(net, graph, name, eps=0.01, conf=0.95, seed=5, max_samples=1 << 36):
    """Time to an answer that meets (eps, conf): plain ELP sizing vs learned sizing, the same bound
    check.  Both arms draw the same estimators (query seed seed + 100, stream 0x51: common random
    numbers), so their difference comes from the sizing and not from the luck of the draws."""
    kind, param, pat = PATTERNS[name]
    prog = Z.Program(kind, param, pat)
    out = {"pattern": name}
    t0 = time.perf_counter()
    elp = Z.elp_plain(graph, prog, eps, conf, seed)
    q = Z.query(graph, prog, eps, conf, max(elp.n_required, 1), seed + 100, stream_id=0x51, max_samples=max_samples)
    out["plain"] = {"n_sized": int(elp.n_required), "samples": int(q.samples), "bound_met": int(q.bound_met),
                    "rel_half_width": q.rel_half_width, "estimate": q.estimate,
                    "seconds": time.perf_counter() - t0, "profile_ms": elp.profile_ms}
    t0 = time.perf_counter()
    q, n = Z.learned_query(net, graph, prog, eps, conf, seed, seed + 100, stream_id=0x51, max_samples=max_samples)
    dt = time.perf_counter() - t0
    _, _, y = Z.learned_budget(net, graph, prog, eps, conf, seed)  # the prediction, for the report (untimed)
    out["learned"] = {"n_sized": int(n), "samples": int(q.samples), "bound_met": int(q.bound_met),
                      "rel_half_width": q.rel_half_width, "estimate": q.estimate,
                      "seconds": dt, "pred_log2_cv2": float(y[0]), "pred_log2_ns": float(y[1])}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--graphs", type=int, default=256)
    ap.add_argument("--heldout", type=int, default=32)
    ap.add_argument("--min-scale", type=int, default=12)
    ap.add_argument("--max-scale", type=int, default=20)
    ap.add_argument("--epochs", type=int, default=400)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--out", default="elp_mlp.npz")
    ap.add_argument("--report", default=None)
    ap.add_argument("--eval-patterns", default="triangle,three_chain,four_chain,four_clique_unbiased,star5")
    ap.add_argument("--eval-cap", type=int, default=1 << 33)
    args = ap.parse_args()
    Z.init(0)
    specs = graph_specs(args.graphs + args.heldout, args.seed, args.min_scale, args.max_scale)
    t0 = time.time()
    X, Y, meta = make_dataset(specs[:args.graphs], log=lambda s: print(s, flush=True))
    net, loss = train(X, Y, seed=args.seed, epochs=args.epochs)
    net.save(args.out)
    pred = net.predict(X)
    rep = {"rows": int(len(X)), "train_seconds": time.time() - t0, "loss_first": float(loss[0]),
           "loss_last": float(np.mean(loss[-50:])), "train_rmse_log2_cv2": float(np.sqrt(np.mean((pred[:, 0] - Y[:, 0]) ** 2)))}
    Xh, Yh, _ = make_dataset(specs[args.graphs:], seed=args.seed + 1)
    ph = net.predict(Xh)
    rep["heldout_rmse_log2_cv2"] = float(np.sqrt(np.mean((ph[:, 0] - Yh[:, 0]) ** 2)))
    rep["heldout_rmse_log2_ns"] = float(np.sqrt(np.mean((ph[:, 1] - Yh[:, 1]) ** 2)))
    rep["heldout_rmse_pilot_only"] = float(np.sqrt(np.mean((Xh[:, 15] - Yh[:, 0]) ** 2)))
    # time to a 1 % / 95 % answer on the held-out graphs: learned vs plain sizing, same bound check
    rows = []
    for spec in specs[args.graphs:]:
        g = build_graph(spec)
        for name in args.eval_patterns.split(","):
            r = compare(net, g, name, eps=0.01, conf=0.95, seed=31, max_samples=args.eval_cap)
            rows.append({"spec": spec, **r})
        g.free()
    sp =[r["plain"]["seconds"] / r["learned"]["seconds"] for r in rows]
    rep["heldout_eval"] = {
        "queries": len(rows), "patterns": args.eval_patterns, "cap": args.eval_cap,
        "bound_met_plain": int(sum(r["plain"]["bound_met"] for r in rows)),
        "bound_met_learned": int(sum(r["learned"]["bound_met"] for r in rows)),
        "median_speedup_learned_over_plain": float(np.median(sp)),
        "learned_faster": int(sum(x > 1 for x in sp)),
        "median_samples_plain": float(np.median([r["plain"]["samples"] for r in rows])),
        "median_samples_learned": float(np.median([r["learned"]["samples"] for r in rows])),
        "by_pattern": {n: {"median_speedup": float(np.median([s for r, s in zip(rows, sp) if r["pattern"] == n])),
                           "bound_met_learned": int(sum(r["learned"]["bound_met"] for r in rows if r["pattern"] == n))}
                       for n in args.eval_patterns.split(",")}}
    print(json.dumps(rep))
    if args.report:
        with open(args.report, "w") as f:
            json.dump({"report": rep, "specs": specs, "meta": meta, "heldout_rows": rows}, f)


if __name__ == "__main__":
    main()
