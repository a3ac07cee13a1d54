"""Generates tests/golden/ from the reference's own code (run here, where the reference exists).

  python tests/golden/make_golden.py        (needs oracle/_ref built by oracle/build_ref.sh)

Per-sample outputs: the reference application's estimate() (compiled from its sources with a
replaying Random) is fed the draws of the oracle's Philox stream; its return values are stored
bit for bit.  Exact counts come from the reference's naive_implementation/ binaries, known
answers from its tests/ programs.  Inputs are the reference's own fixture graphs (small-10,
simple-30, wiki-vote) and seeded synthetic graphs from zg_gen_* (stored as parameters plus a
checksum, regenerated by the tests).
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "sampling-graph-mining_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
REF = os.environ.get("ZG_REFERENCE_DIR", "/root/reference")

import oracle as O  # noqa: E402
import zgraph as Z  # noqa: E402

STAR = (5, [(0, 1), (0, 2), (0, 3), (0, 4)])
HOUSE = (5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)])
TRI = (3, [(0, 1), (0, 2), (1, 2)])

# (label, reference driver, program kind, param, pattern)
PROGRAMS = [
    ("triangle", "triangle", Z.PROG_TRIANGLE, 0, None),
    ("four_clique", "four_clique", Z.PROG_FOUR_CLIQUE, 0, None),
    ("three_chain", "three_chain", Z.PROG_THREE_CHAIN, 0, None),
    ("four_chain", "four_chain", Z.PROG_FOUR_CHAIN, 0, None),
    ("chain4", "chain", Z.PROG_CHAIN, 4, None),
    ("chain6", "chain", Z.PROG_CHAIN, 6, None),
    ("star", "pattern", Z.PROG_PATTERN, 0, STAR),
    ("house", "pattern", Z.PROG_PATTERN, 0, HOUSE),
    ("tri_pattern", "pattern", Z.PROG_PATTERN, 0, TRI),
]

SYNTHETIC = {
    "rmat10": ("rmat", dict(scale=10, edge_factor=8, a=0.57, b=0.19, c=0.19, seed=3), 1 << 10),
    "dense7": ("rmat", dict(scale=7, edge_factor=30, a=0.45, b=0.2, c=0.2, seed=2), 1 << 7),
    "chunglu3k": ("chung_lu", dict(n=3000, exponent=2.3, avg_degree=12.0, seed=9), 3000),
}
NAIVE = {"triangle": "TriangleCounting", "wedge": "ThreeChain", "three_path": "FourChain",
         "five_star": "FiveStar", "four_clique": "FourClique", "five_chain": "FiveChain",
         "house": "FiveHouse"}


def synth(name):
    kind, p, nv = SYNTHETIC[name]
    if kind == "rmat":
        e = Z.gen_rmat(p["scale"], p["edge_factor"], p["a"], p["b"], p["c"], p["seed"])
    else:
        e = Z.gen_chung_lu(p["n"], p["exponent"], p["avg_degree"], p["seed"])
    return e, nv


def checksum(e):
    return hashlib.sha256(np.ascontiguousarray(e, dtype=np.uint32).tobytes()).hexdigest()


def read_edgelist(path):
    with open(path) as f:
        nv, m = map(int, f.readline().split())
        rows = [list(map(int, line.split())) for line in f if line.strip()]
    a = np.array(rows[:m], dtype=np.uint32)
    return a, nv


def naive(bin_name, edges, nv, weights=None):
    with tempfile.NamedTemporaryFile("w", suffix=".edgelist", delete=False) as f:
        f.write("%d %d\n" % (nv, len(edges)))
        for i, (s, d) in enumerate(edges):
            if weights is None:
                f.write("%d %d\n" % (s, d))
            else:
                f.write("%d %d %d\n" % (s, d, weights[i]))
        path = f.name
    try:
        out = subprocess.run([os.path.join(O.REF_DIR, "bin", "naive_" + bin_name), path], capture_output=True,
                             text=True, timeout=600).stdout
    finally:
        os.unlink(path)
    line = [x for x in out.replace("\x1b[F", "\n").splitlines() if x.startswith("count:")][-1]
    return int(line.split()[1])


def main():
    if not O.ref_available():
        sys.exit("oracle/_ref is not built (run oracle/build_ref.sh)")
    Z.lib()
    graphs = {}
    small10, nv10 = read_edgelist(os.path.join(REF, "datasets/small-10/small-10.edgelist"))
    simple30, nv30 = read_edgelist(os.path.join(REF, "datasets/simple-30/dataset/simple-30.edgelist"))
    wiki, nvw = read_edgelist(os.path.join(REF, "datasets/wiki-vote/dataset/wiki-vote.edgelist"))
    wikiw, _ = read_edgelist(os.path.join(REF, "datasets/wiki-vote/dataset/wiki-vote.weighted.edgelist"))
    graphs["small10"] = (small10, nv10)
    graphs["simple30"] = (simple30, nv30)
    graphs["wiki_vote"] = (wiki, nvw)
    for name in SYNTHETIC:
        graphs[name] = synth(name)

    arrays = {"small10_edges": small10, "simple30_edges": simple30,
              "wiki_vote_edges": wiki, "wiki_vote_weights": wikiw[:, 2].copy()}
    meta = {"graphs": {}, "samples": {}, "naive": {}, "kat": {}, "elp": {}}
    for name, (e, nv) in graphs.items():
        meta["graphs"][name] = {"num_vertices": nv, "m": int(len(e)), "sha256": checksum(e)}
        if name in SYNTHETIC:
            meta["graphs"][name]["generator"] = SYNTHETIC[name][0]
            meta["graphs"][name]["params"] = SYNTHETIC[name][1]

    # per-sample outputs of the reference estimators
    n, seed, stream = 3000, 1234, 7
    for gname in ("small10", "simple30", "rmat10", "dense7", "chunglu3k", "wiki_vote"):
        e, nv = graphs[gname]
        og = O.OracleGraph(e, nv)
        for label, app, kind, param, pat in PROGRAMS:
            op = O.OracleProgram(kind, param, pat)
            tr, _ = O.traces(og, op, n, seed, stream=stream)
            ri = O.RefInstance(app, e, nv, param=param, pattern=pat)
            out, used, bad = ri.estimates(tr)
            ri.close()
            assert bad == 0, (gname, label, bad)
            key = "%s__%s" % (gname, label)
            arrays["w__" + key] = out.view(np.uint64)
            arrays["ndraws__" + key] = used
            meta["samples"][key] = {"n": n, "seed": seed, "stream": stream, "kind": kind, "param": param,
                                    "pattern": pat, "hits": int(np.count_nonzero(out))}
        # calculate() of the triangle instance: the reference's own reduction
        op = O.OracleProgram(Z.PROG_TRIANGLE)
        tr, _ = O.traces(og, op, n, seed, stream=stream)
        ri = O.RefInstance("triangle", e, nv)
        r, bad = ri.calculate(tr)
        ri.close()
        assert bad == 0
        meta["samples"]["%s__triangle" % gname]["calculate"] = r.hex()
        # ThreeMotif: chain estimators + triangle estimators re-closing their wedges
        tc, tt, _, _ = O.three_motif(og, 2000, n, seed, 1, 2)
        a, b, bad = O.ref_motif(e, nv, 2000, n, tc, tt)
        assert bad == 0
        meta["samples"]["%s__three_motif" % gname] = {"n_chain": 2000, "n_tri": n, "seed": seed, "stream_chain": 1,
                                                      "stream_tri": 2, "chain": a.hex(), "triangle": b.hex()}

    # AllPredicate weighted triangle on wiki-vote's weights (w >= 50 and the inverted w < 50)
    e, nv = graphs["wiki_vote"]
    w = arrays["wiki_vote_weights"]
    for op_code, t, sh in ((Z.PRED_GE, 50, 4242), (Z.PRED_LT, 50, 4343), (Z.PRED_GE, 30, 4444)):
        idx = np.nonzero(np.array([O.pred(op_code, t, 0, int(x)) for x in w]))[0]
        perm = O.shuffle_perm(len(idx), sh)
        fe = e[idx][perm.astype(np.int64)]
        ogf = O.OracleGraph(fe, nv)
        tr, _ = O.traces(ogf, O.OracleProgram(Z.PROG_TRIANGLE), n, seed, stream=stream)
        ri = O.RefInstance("pred_triangle", e, nv, weights=w, param=(op_code << 24) | t, filter_perm=perm)
        out, used, bad = ri.estimates(tr)
        ri.close()
        assert bad == 0
        key = "wiki_vote__pred_%d_%d" % (op_code, t)
        arrays["w__" + key] = out.view(np.uint64)
        meta["samples"][key] = {"n": n, "seed": seed, "stream": stream, "op": op_code, "t": t, "shuffle_seed": sh,
                                "filtered_m": int(len(idx)), "hits": int(np.count_nonzero(out))}

    # ErrorProfile::get_num_estimators of the reference, replaying the zg_elp_plain draw plan
    meta["elp"]["get_num_estimators"] = []
    for gname, app, kind, param, seed in (("rmat10", "triangle", Z.PROG_TRIANGLE, 0, 77),
                                          ("rmat10", "three_chain", Z.PROG_THREE_CHAIN, 0, 78),
                                          ("dense7", "four_chain", Z.PROG_FOUR_CHAIN, 0, 79),
                                          ("dense7", "chain", Z.PROG_CHAIN, 5, 80)):
        e, nv = graphs[gname]
        n_req, bad = O.ref_elp(app, e, nv, kind, param=param, seed=seed, eps=0.05, conf=0.95)
        assert bad == 0, (gname, app)
        meta["elp"]["get_num_estimators"].append({"graph": gname, "kind": kind, "param": param, "seed": seed,
                                                  "eps": 0.05, "conf": 0.95, "n_required": n_req})

    # exact counts from naive_implementation/
    for gname in ("small10", "simple30", "rmat10", "dense7", "chunglu3k", "wiki_vote"):
        e, nv = graphs[gname]
        counts = {}
        for kind, bin_name in NAIVE.items():
            if gname in ("wiki_vote", "chunglu3k") and kind in ("four_clique", "five_chain", "house"):
                continue
            if kind == "five_chain" and nv < 10:
                continue  # FiveChain.cpp:47 takes v_0 % (vertices / 10): division by zero below 10 vertices
            counts[kind] = naive(bin_name, e, nv)
        meta["naive"][gname] = counts
    e, nv = graphs["wiki_vote"]
    meta["naive"]["wiki_vote"]["weighted_triangle_50"] = naive("WeightedTriangleCounting", e, nv, w)
    meta["naive"]["wiki_vote"]["at_least_one_triangle_50"] = naive("AtLeastOneWeightedTriangleCounting", e, nv, w)

    # known answers printed by the reference's tests/ programs
    def run_test(t):
        return subprocess.run([os.path.join(O.REF_DIR, "bin", t)], capture_output=True, text=True).stdout
    meta["kat"]["TestRegression"] = run_test("TestRegression").strip()
    meta["kat"]["TestSubgraph"] = run_test("TestSubgraph").strip().splitlines()[-1]
    meta["kat"]["TestPattern"] = [x for x in run_test("TestPattern").splitlines() if "/" in x and x[0].isdigit()]
    meta["kat"]["TestPattern2"] = [x for x in run_test("TestPattern2").splitlines() if "/" in x and x[0].isdigit()]

    # ELP building blocks through the reference's own functions
    rng = np.random.default_rng(5)
    L = O.ref_lib("pattern")
    reg = []
    for _ in range(20):
        k = int(rng.integers(1, 200))
        x = rng.random(k) * 10
        y = rng.random(k)
        xs, ys = np.ascontiguousarray(x), np.ascontiguousarray(y)
        reg.append({"x": x.tolist(), "y": y.tolist(), "k": L.zgref_regression_k(O._p(xs), O._p(ys), k).hex()})
    meta["elp"]["regression"] = reg
    bounds = []
    for _ in range(50):
        args = (float(rng.uniform(0.001, 1)), float(rng.uniform(0.001, 0.5)), 1.0, float(rng.integers(1, 6)),
                float(rng.uniform(1, 1e9)), int(rng.integers(1, 10**6)), int(rng.integers(1, 10**9)))
        bounds.append({"args": list(args), "bound": L.zgref_calculate_bound(*args).hex()})
    meta["elp"]["calculate_bound"] = bounds
    folds = []
    for _ in range(10):
        k = int(rng.integers(1, 50))
        ns = rng.integers(1, 1 << 20, size=k).astype(np.uint64)
        vals = rng.random(k) * 1e6
        folds.append({"n": ns.tolist(), "v": vals.tolist(),
                      "r": L.zgref_estimation_fold(O._p(ns), O._p(np.ascontiguousarray(vals)), k).hex()})
    meta["elp"]["estimation_fold"] = folds

    np.savez_compressed(os.path.join(HERE, "reference_outputs.npz"), **arrays)
    with open(os.path.join(HERE, "reference_outputs.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "reference_outputs.npz"))


if __name__ == "__main__":
    main()
