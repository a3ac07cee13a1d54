"""The CPU oracle against outputs the reference's own code produced (tests/golden/, made by
tests/golden/make_golden.py): per-sample estimate() values bit for bit, calculate()'s reduction,
ThreeMotif's cached run, the all-predicate triangle on a filtered graph, naive exact counts,
the reference tests' known answers and the ELP building blocks."""
import json
import os

import numpy as np
import pytest

import oracle as O
import zgraph as Z
from conftest import GOLDEN

STAR = (5, [(0, 1), (0, 2), (0, 3), (0, 4)])
HOUSE = (5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)])
TRI = (3, [(0, 1), (0, 2), (1, 2)])


@pytest.fixture(scope="module")
def golden():
    meta = json.load(open(os.path.join(GOLDEN, "reference_outputs.json")))
    arr = np.load(os.path.join(GOLDEN, "reference_outputs.npz"))
    return meta, arr


def golden_graph(meta, arr, name):
    g = meta["graphs"][name]
    if name + "_edges" in arr:
        e = arr[name + "_edges"]
    elif g["generator"] == "rmat":
        p = g["params"]
        e = Z.gen_rmat(p["scale"], p["edge_factor"], p["a"], p["b"], p["c"], p["seed"])
    else:
        p = g["params"]
        e = Z.gen_chung_lu(p["n"], p["exponent"], p["avg_degree"], p["seed"])
    import hashlib
    assert hashlib.sha256(np.ascontiguousarray(e, dtype=np.uint32).tobytes()).hexdigest() == g["sha256"]
    return e, g["num_vertices"]


def test_samples_bit_exact(golden):
    meta, arr = golden
    graphs = {}
    checked = 0
    for key, s in meta["samples"].items():
        gname, label = key.split("__")
        if label == "three_motif" or label.startswith("pred_"):
            continue
        if gname not in graphs:
            e, nv = golden_graph(meta, arr, gname)
            graphs[gname] = O.OracleGraph(e, nv)
        pat = s["pattern"]
        prog = O.OracleProgram(s["kind"], s["param"], None if pat is None else (pat[0], pat[1]))
        tr, _ = O.traces(graphs[gname], prog, s["n"], s["seed"], stream=s["stream"])
        assert np.array_equal(tr["w"].view(np.uint64), arr["w__" + key]), key
        assert np.array_equal(tr["ndraws"], arr["ndraws__" + key]), key
        checked += 1
        if "calculate" in s:
            # calculate(n): one thread sums estimate() in sample order, divides by n (:273-292)
            acc = 0.0
            for w in tr["w"]:
                acc += w
            assert (acc / float(s["n"])).hex() == s["calculate"]
    assert checked >= 50


def test_three_motif(golden):
    meta, arr = golden
    for key, s in meta["samples"].items():
        gname, label = key.split("__")
        if label != "three_motif":
            continue
        e, nv = golden_graph(meta, arr, gname)
        tc, tt, _, _ = O.three_motif(O.OracleGraph(e, nv), s["n_chain"], s["n_tri"], s["seed"], s["stream_chain"],
                                     s["stream_tri"])
        for tr, n, ref in ((tc, s["n_chain"], s["chain"]), (tt, s["n_tri"], s["triangle"])):
            acc = 0.0
            for w in tr["w"]:
                acc += w
            assert (acc / float(n)).hex() == ref, key


def test_all_predicate_triangle(golden):
    meta, arr = golden
    e, nv = golden_graph(meta, arr, "wiki_vote")
    w = arr["wiki_vote_weights"]
    for key, s in meta["samples"].items():
        if "__pred_" not in key:
            continue
        keep = np.array([O.pred(s["op"], s["t"], 0, int(x)) for x in w])
        idx = np.nonzero(keep)[0]
        assert len(idx) == s["filtered_m"]
        fe = e[idx][O.shuffle_perm(len(idx), s["shuffle_seed"]).astype(np.int64)]
        tr, _ = O.traces(O.OracleGraph(fe, nv), O.OracleProgram(Z.PROG_TRIANGLE), s["n"], s["seed"],
                         stream=s["stream"])
        assert np.array_equal(tr["w"].view(np.uint64), arr["w__" + key]), key


def test_naive_exact_counts(golden):
    meta, arr = golden
    kinds = {"triangle": Z.EXACT_TRIANGLE, "wedge": Z.EXACT_WEDGE, "three_path": Z.EXACT_THREE_PATH,
             "five_star": Z.EXACT_FIVE_STAR, "four_clique": Z.EXACT_FOUR_CLIQUE, "house": Z.EXACT_FIVE_HOUSE,
             "five_chain": Z.EXACT_FIVE_CHAIN}
    weighted = {"weighted_triangle_50", "at_least_one_triangle_50"}
    checked = set()
    for gname, counts in meta["naive"].items():
        e, nv = golden_graph(meta, arr, gname)
        og = O.OracleGraph(e, nv)
        for k, v in counts.items():
            assert k in kinds or k in weighted, "golden count %s has no check" % k
            if k in kinds:
                assert og.exact_fast(kinds[k]) == v, (gname, k)
                checked.add(k)
                # the naive walks enumerate every path one by one: only where that stays quick
                slow = (gname == "wiki_vote" and k == "three_path") or (k == "four_clique" and nv > 4096) or \
                       (k in ("house", "five_chain") and v > 10 ** 8)
                if not slow:
                    assert og.exact_naive(kinds[k]) == v, (gname, k)
    assert checked == set(kinds)
    e, nv = golden_graph(meta, arr, "wiki_vote")
    og = O.OracleGraph(e, nv, arr["wiki_vote_weights"])
    assert og.exact_weighted_triangle(50, False) == meta["naive"]["wiki_vote"]["weighted_triangle_50"]
    assert og.exact_weighted_triangle(50, True) == meta["naive"]["wiki_vote"]["at_least_one_triangle_50"]


def test_known_answers(golden):
    meta, _ = golden
    kat = meta["kat"]
    # tests/TestPattern2.cpp: unique vertex relabelings of the 4-chain, 4-clique and 5-star
    chain4 = (4, [(0, 1), (1, 2), (2, 3)])
    clique4 = (4, [(1, 0), (2, 0), (2, 1), (3, 0), (3, 1), (3, 2)])
    got = []
    for nv, edges in (chain4, clique4, STAR):
        p = O.OracleProgram(Z.PROG_PATTERN, 0, (nv, edges))
        fact = int(np.prod(np.arange(1, nv + 1)))
        got.append("%d/%d" % (p.num_unique, fact))
    assert got == kat["TestPattern2"]
    # tests/TestRegression.cpp: k^2 of the fixed arrays
    te = np.array([0.09, 0.26, 0.15, 0.42, 0.57, 0.10, 2.62]) / 100.0
    ee = np.array([1, 2, 4, 8, 16, 32, 64], dtype=np.float64) / 100.0
    k = O.regression_k(te, ee)
    assert "%.4f" % (k * k) == kat["TestRegression"]
    assert kat["TestSubgraph"].endswith("1<->2)")


def test_elp_building_blocks(golden):
    meta, _ = golden
    for c in meta["elp"]["regression"]:
        assert O.regression_k(np.array(c["x"]), np.array(c["y"])).hex() == c["k"]
    for c in meta["elp"]["calculate_bound"]:
        a = c["args"]
        assert O.calculate_bound(a[0], a[1], a[2], a[3], a[4], int(a[5]), int(a[6])).hex() == c["bound"]
    for c in meta["elp"]["estimation_fold"]:
        e = Z.Estimation()
        for n, v in zip(c["n"], c["v"]):
            e.update(n, v)
        assert e.get_currnet_estimation().hex() == c["r"]


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32 with 10 rounds
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert O.philox([0xffffffff] * 4, [0xffffffff] * 2) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert O.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_x87_emulation_matches_long_double():
    import ctypes
    import platform
    rng = np.random.default_rng(1)
    for _ in range(2000):
        k = int(rng.integers(1, 12))
        f = rng.integers(1, 1 << 20, size=k).astype(np.float64)
        f = 1.0 / f * rng.integers(1, 3, size=k)
        got = O.ext_inv_product(f)
        if platform.machine() in ("x86_64", "AMD64") and ctypes.sizeof(ctypes.c_longdouble) == 16:
            p = np.longdouble(1.0)
            for x in f:
                p = p * np.longdouble(x)
            assert got == float(np.longdouble(1.0) / p)
        assert abs(got * np.prod(f) - 1.0) < 1e-12


def test_error_profile_matches_reference(golden):
    """zg_elp_solve on the oracle's draws of the zg_elp_plain plan reproduces the reference's own
    ErrorProfile::get_num_estimators (src/ErrorLatencyProfile.cpp:72-207)."""
    meta, arr = golden
    for case in meta["elp"]["get_num_estimators"]:
        e, nv = golden_graph(meta, arr, case["graph"])
        seed = case["seed"]
        keep = np.array([O.subsample_keep(0.1, seed + Z.ELP_KEEP_OFFSET, i) for i in range(len(e))])
        kept = np.nonzero(keep)[0]
        sub = e[kept[O.shuffle_perm(len(kept), seed + Z.ELP_SHUFFLE_OFFSET).astype(np.int64)]]
        og = O.OracleGraph(sub, nv)
        prog = O.OracleProgram(case["kind"], case["param"])
        tr, _ = O.traces(og, prog, 1 << 18, seed, stream=Z.ELP_STREAM)
        groups = []
        for row in tr["w"].reshape(-1, 16):
            acc = 0.0
            for x in row:
                acc += float(x)
            groups.append(acc / 16.0)
        big = O.run(og, prog, 1 << 23, seed, Z.ELP_STREAM, 1 << 18)
        ncse = {Z.PROG_TRIANGLE: 1, Z.PROG_THREE_CHAIN: 1, Z.PROG_FOUR_CHAIN: 2,
                Z.PROG_CHAIN: case["param"] - 2}[case["kind"]]
        r = Z.elp_solve(np.array(groups), 16, float(big.exact_sum() / big.samples), 1 << 23, 1.0, float(ncse),
                        len(sub), int(np.bincount(sub.ravel(), minlength=nv).max()), len(e),
                        int(np.bincount(e.ravel(), minlength=nv).max()), case["eps"], case["conf"])
        assert abs(r.n_required - case["n_required"]) <= 1e-9 * case["n_required"] + 1, (case, r.n_required)


def test_oracle_unbiased_four_clique_matches_exact_counts():
    """The canonical-path 4-clique program (no counterpart in the reference) is unbiased: on three
    graphs its mean over 2^21 samples lies within 4 standard errors of the exact count, while the
    reference's FourClique estimate is about 0.6 of it."""
    import math
    import zgraph as Z
    for sc, ef, seed in ((8, 16, 3), (9, 12, 5), (7, 24, 8)):
        e = Z.gen_rmat(sc, ef, seed=seed)
        og = O.OracleGraph(e, 1 << sc)
        ex = og.exact_naive(5)
        c = O.run(og, O.OracleProgram(7), 1 << 21, 11, stream=7)
        n = c.samples
        mean = float(c.exact_sum()) / n
        se = math.sqrt(max(c.sum_w2 / n - mean * mean, 0.0) / n)
        assert abs(mean - ex) < 4 * se, (sc, ef, mean, ex, se)
        r = O.run(og, O.OracleProgram(2), 1 << 21, 11, stream=2)
        assert float(r.exact_sum()) / r.samples < 0.75 * ex


def test_subsample_edges_matches_the_per_edge_plan(golden):
    """zgo_subsample_edges (parallel keep draws and radix-sorted shuffle keys) returns the edge list
    that the per-edge keep draws and zgo_shuffle_perm give, in the same order."""
    import zgraph as Z
    meta, arr = golden
    for name in sorted(meta["graphs"])[:3]:
        e, nv = golden_graph(meta, arr, name)
        for seed in (1, 77):
            keep = np.array([O.subsample_keep(0.1, seed + 1, i) for i in range(len(e))], dtype=bool)
            kept = np.nonzero(keep)[0]
            want = e[kept[O.shuffle_perm(len(kept), seed + 2).astype(np.int64)]]
            got = O.subsample_edges(e, 0.1, seed + 1, seed + 2)
            assert np.array_equal(got, want), (name, seed)
    assert (O.ELP_KEEP_OFFSET, O.ELP_SHUFFLE_OFFSET, O.ELP_FILTER_OFFSET, O.ELP_STREAM) == \
        (Z.ELP_KEEP_OFFSET, Z.ELP_SHUFFLE_OFFSET, Z.ELP_FILTER_OFFSET, Z.ELP_STREAM)


def test_host_plain_elp_matches_reference(golden):
    """The host restatement of ErrorProfile::get_num_estimators (oracle.plain_elp, which the CPU
    arm of the benchmark times without the GPU library) gives the reference's own estimator count
    on every golden case."""
    meta, arr = golden
    ncse_of = {1: 1, 3: 1, 4: 2}
    for case in meta["elp"]["get_num_estimators"]:
        e, nv = golden_graph(meta, arr, case["graph"])
        ncse = ncse_of.get(case["kind"], case["param"] - 2)
        deg = np.bincount(e.ravel(), minlength=nv)
        n = O.plain_elp(e, nv, O.OracleProgram(case["kind"], case["param"]), ncse, case["seed"], case["eps"],
                        case["conf"], len(e), int(deg.max()))
        assert abs(n - case["n_required"]) <= 1e-9 * case["n_required"] + 1, (case, n)


def test_device_elp_solve_matches_host_restatement_on_random_profiles():
    """zg_elp_solve (the host half of zg_elp_plain, in the product library) and the oracle's own
    restatement of ErrorProfile::get_num_estimators's host half agree on random group-estimate
    sequences: heavy-tailed and light-tailed group means, zero groups, several program shapes
    (sample_edge / conditional_sample_edge call counts) and error / confidence targets."""
    import zgraph as Z
    rng = np.random.default_rng(2024)
    for trial in range(24):
        n_groups = int(rng.choice([64, 1024, 1 << 14]))
        mean = float(10 ** rng.uniform(2, 9))
        if trial % 3 == 0:
            groups = rng.pareto(1.5, n_groups) * mean
        else:
            groups = rng.gamma(2.0, mean / 2.0, n_groups)
        groups[rng.random(n_groups) < 0.2] = 0.0
        big = float(groups.mean() * rng.uniform(0.8, 1.2))
        ncse = float(rng.integers(1, 5))
        sm, sd = int(rng.integers(10 ** 4, 10 ** 7)), int(rng.integers(10, 10 ** 4))
        om, od = sm * 10, sd * int(rng.integers(2, 12))
        eps, conf = float(rng.choice([0.01, 0.05, 0.1])), float(rng.choice([0.9, 0.95, 0.99]))
        want = O.elp_solve(groups, 16, big, 1 << 23, 1.0, ncse, sm, sd, om, od, eps, conf)
        got = Z.elp_solve(groups, 16, big, 1 << 23, 1.0, ncse, sm, sd, om, od, eps, conf)
        assert abs(got.n_required_f - want) <= 1e-9 * abs(want), (trial, got.n_required_f, want)


def test_untraced_and_traced_runs_give_the_same_counters():
    """An oracle run that keeps no per-sample trace (per-thread counters, no access model) returns
    the counters of the traced run of the same samples, for every program kind, with 1 and 4
    threads: the checker the GPU parity tests compare against is the same either way."""
    import zgraph as Z
    e = Z.gen_rmat(11, 12, seed=4)
    og = O.OracleGraph(e, 1 << 11)
    progs = [O.OracleProgram(k) for k in (1, 2, 3, 4, 7)] + [O.OracleProgram(5, 6)]
    progs += [O.OracleProgram(6, pattern=(5, [(0, 1), (0, 2), (0, 3), (0, 4)])),
              O.OracleProgram(6, pattern=(5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)]))]
    for p in progs:
        _, want = O.traces(og, p, 1 << 15, 99, stream=3, first=1 << 33)
        for threads in (1, 4):
            got = O.run(og, p, 1 << 15, 99, 3, 1 << 33, threads)
            for f in ("samples", "hits", "fails", "den_log2", "overflow"):
                assert getattr(got, f) == getattr(want, f), (p.p.kind, threads, f)
            assert list(got.sum_num) == list(want.sum_num) and got.estimate == want.estimate, (p.p.kind, threads)
            assert got.sum_w2 == pytest.approx(want.sum_w2, rel=1e-12), (p.p.kind, threads)
