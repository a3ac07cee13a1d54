"""The learned error-latency profile: the network's forward, backward and Adam kernels against the
CPU oracle (oracle/mlp_oracle.py), training convergence, the query features, and what the
trained network gains over plain ErrorProfile sizing on held-out graphs."""
import math

import numpy as np
import pytest

import mlp_oracle as M
import zgraph as Z

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _init():
    Z.init(0)


def test_gradient_matches_oracle():
    rng = np.random.default_rng(1)
    for seed in (5, 6, 7):
        net = Z.Mlp(seed)
        params, _ = net.params()
        for B in (1, 17, 64):
            X = rng.normal(size=(B, 16)).astype(np.float32)
            Y = rng.normal(size=(B, 2)).astype(np.float32)
            g, loss = net.grad(X, Y)
            loss_ref, g_ref = M.loss_and_grad(params, X, Y)
            assert abs(loss - loss_ref) <= 1e-5 * max(1.0, loss_ref)
            scale = np.abs(g_ref).max()
            assert np.allclose(g, g_ref, rtol=2e-3, atol=1e-5 * scale), np.abs(g - g_ref).max() / scale


def test_adam_step_matches_oracle():
    rng = np.random.default_rng(2)
    net = Z.Mlp(9)
    p0, _ = net.params()
    X = rng.normal(size=(64, 16)).astype(np.float32) * 3 + 1
    Y = rng.normal(size=(64, 2)).astype(np.float32) * 2 - 1
    lr = 1e-3
    net.train(X, Y, epochs=1, batch=64, lr=lr, seed=1)
    p1, norm = net.params()
    # the device normalised with float64 mean / population std, stored as float32
    xm, xs, ym, ys = norm[:16], norm[16:32], norm[32:34], norm[34:36]
    assert np.allclose(xm, X.astype(np.float64).mean(0), rtol=1e-5, atol=1e-6)
    Xn = ((X - xm) / xs).astype(np.float32)
    Yn = ((Y - ym) / ys).astype(np.float32)
    _, g = M.loss_and_grad(p0, Xn, Yn)
    pr, _, _ = M.adam_step(p0.astype(np.float64), np.zeros(M.NP), np.zeros(M.NP), g, 1, lr)
    big = np.abs(g) > 1e-5
    assert big.sum() > 4000
    assert np.allclose(p1[big], pr[big], rtol=0, atol=lr * 1e-2)


def test_predict_matches_oracle():
    rng = np.random.default_rng(3)
    net = Z.Mlp(4)
    X = rng.normal(size=(500, 16)).astype(np.float32)
    Y = rng.normal(size=(500, 2)).astype(np.float32)
    net.train(X, Y, epochs=2, batch=50, lr=1e-3)
    params, norm = net.params()
    got = net.predict(X)
    y, _ = M.forward(params, (X - norm[:16]) / norm[16:32])
    ref = y * norm[34:36] + norm[32:34]
    assert np.allclose(got, ref, rtol=1e-4, atol=1e-4)


def test_training_reduces_loss():
    rng = np.random.default_rng(4)
    X = rng.normal(size=(2048, 16)).astype(np.float32)
    Y = np.stack([np.sin(X[:, 0]) + 0.5 * X[:, 1] ** 2, X[:, 2] * X[:, 3] - X[:, 4]], 1).astype(np.float32)
    net = Z.Mlp(8)
    loss = net.train(X, Y, epochs=60, batch=64, lr=3e-3)
    assert loss[-50:].mean() < 0.1 * loss[:50].mean()
    pred = net.predict(X)
    assert np.mean((pred - Y) ** 2) < 0.1 * np.var(Y)


def test_features_match_host():
    e = Z.gen_rmat(11, 8, seed=7)
    nv = 1 << 11
    g = Z.Graph.from_edges(e, nv)
    f = Z.features(g, Z.Program(Z.PROG_TRIANGLE), 1 << 16, 3)
    d = np.bincount(e.ravel(), minlength=nv).astype(np.float64)
    nz = d[d > 0]
    m = len(e)
    du, dv = d[e[:, 0]], d[e[:, 1]]
    want = [math.log2(m), math.log2(len(nz)), math.log2(nz.max()), math.log2(nz.mean()),
            math.log2((nz ** 2).mean()), math.log2((nz ** 3).mean()), math.log2((du + dv).mean()),
            math.log2(np.minimum(du, dv).mean())]
    assert np.allclose(f[:8], want, rtol=1e-5)
    assert list(f[8:14]) == [1, 0, 0, 0, 0, 0]
    c = Z.Program(Z.PROG_TRIANGLE).run(g, 1 << 16, 3, stream_id=Z.ELP_STREAM + 1)
    assert abs(f[14] - math.log2((c.hits + 0.5) / (1 << 16))) < 1e-5


def test_adaptive_pilot():
    """pilot_samples = 0: the features of the first pilot in 2^16, 2^18, 2^20, 2^22 with 8 hits (the
    last if none has), each pilot from the pilot stream's first sample."""
    e = Z.gen_rmat(12, 3, seed=21)
    g = Z.Graph.from_edges(e, 1 << 12)
    for kind in (Z.PROG_TRIANGLE, Z.PROG_FOUR_CLIQUE, Z.PROG_FOUR_CLIQUE_UNBIASED):
        p = Z.Program(kind)
        f0 = Z.features(g, p, 0, 5)
        for n in (1 << 16, 1 << 18, 1 << 20, 1 << 22):
            if p.run(g, n, 5, stream_id=Z.ELP_STREAM + 1).hits >= 8 or n == 1 << 22:
                break
        assert np.array_equal(f0, Z.features(g, p, n, 5)), (kind, n)


def test_learned_budget_and_query_entry_points():
    """zg_elp_learned is the sizing formula on the network's prediction for the query's features;
    zg_query_learned runs it and checks the answer's bound, half of a long budget first."""
    e = Z.gen_rmat(12, 10, seed=8)
    g = Z.Graph.from_edges(e, 1 << 12)
    net = Z.Mlp(5)
    rng = np.random.default_rng(6)
    net.train(rng.normal(size=(128, 16)).astype(np.float32), rng.normal(size=(128, 2)).astype(np.float32) + 6,
              epochs=2, batch=32, lr=1e-3)
    p = Z.Program(Z.PROG_TRIANGLE)
    n, f, y = Z.learned_budget(net, g, p, 0.02, 0.95, seed=4)
    y_ref = net.predict(f[None, :])[0]
    assert np.allclose(y, y_ref, rtol=1e-6, atol=1e-6)
    z = Z.lib().zg_normal_quantile(0.975)
    assert n == max(int(z * z * 2.0 ** float(y_ref[0]) / 0.02 ** 2), 1 << 16)
    q, n2 = Z.learned_query(net, g, p, 0.02, 0.95, 4, 77, stream_id=3, max_samples=1 << 32)
    assert n2 == n and q.bound_met and q.rel_half_width <= 0.02
    # the first round of the bound check ran the budget (below 2^30: one look), continued from the same stream
    first = Z.query(g, p, 0.02, 0.95, n, 77, stream_id=3, max_samples=1 << 32)
    assert (q.samples, q.estimate) == (first.samples, first.estimate)


def test_learned_sizing_beats_plain_elp():
    """Trained on small synthetic graphs, the network sizes held-out queries far closer to what the
    empirical bound needs than ErrorProfile does; both deliver answers that meet the bound."""
    import elp_learn as EL
    specs = EL.graph_specs(18, 99, min_scale=9, max_scale=12, edge_factor=(4, 12))
    pats = {k: EL.PATTERNS[k] for k in ("triangle", "three_chain", "four_chain", "star5")}
    X, Y, _ = EL.make_dataset(specs[:14], patterns=pats, seed=5)
    assert len(X) >= 40
    net, loss = EL.train(X, Y, seed=3, epochs=300)
    assert loss[-20:].mean() < loss[:20].mean()
    wins, rows = 0, []
    for spec in specs[14:]:
        g = EL.build_graph(spec)
        for name in ("triangle", "three_chain", "four_chain"):
            r = EL.compare(net, g, name, eps=0.05, conf=0.95, seed=21, max_samples=1 << 34)
            rows.append(r)
            assert r["plain"]["bound_met"] and r["learned"]["bound_met"], r
            wins += r["learned"]["samples"] < r["plain"]["samples"]
    assert wins >= 0.8 * len(rows), rows
    t_plain = np.median([r["plain"]["seconds"] for r in rows])
    t_learned = np.median([r["learned"]["seconds"] for r in rows])
    assert t_learned < t_plain, (t_learned, t_plain)
