"""Learned null on the device: features and the network's forward pass and
gradient against the CPU oracle, training behaviour, and the learned-null
E-values against the gamma tail they come from."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NRM_ID = np.concatenate([np.zeros(64), np.ones(64), np.zeros(3), np.ones(3)]).astype(np.float32)


@pytest.mark.parametrize("N,L,weights", [(40, 77, "unit"), (300, 160, "gsc"), (1200, 64, "pb")])
def test_features_match_oracle(covgpu, oracle, N, L, weights):
    s = covgpu.Synth(N, L, 1.2, 10, 2, 5, 5, 0.1, seed=N + L)
    e = covgpu.Engine(N, L)
    e.set_alignment(0, s.ax)
    if weights == "unit":
        w = np.ones(N)
        e.set_weights(w)
    elif weights == "gsc":
        w = e.weights_gsc(0, set=True)
    else:
        w = e.weights_pb(0, set=True)
    got = e.features(0, 0.9)
    ref = oracle.features(s.ax, w, 0.9)
    e.close()
    assert np.all(np.isfinite(got))
    sc = np.r_[0:5, 37:47]
    assert np.allclose(got[sc], ref[sc], rtol=2e-6, atol=1e-6), np.abs(got[sc] - ref[sc]).max()
    assert np.all(got[47:] == 0.0)
    # histogram fractions: a value on a bin edge may land in the neighbour
    # after a last-bit difference of the summation order, at most one count
    for q in range(2):
        d = np.abs(got[5 + 16 * q: 21 + 16 * q] - ref[5 + 16 * q: 21 + 16 * q]) * L
        assert d.sum() <= 2.01, (q, d)


def test_quick_null_summary(covgpu):
    """Features 47-63: the score summary of the quick nulls, consistent with
    covgpu_rscape run on the same nulls."""
    N, L, nq = 150, 90, 4
    s = covgpu.Synth(N, L, 1.5, 15, 2, 7, 8, 0.08, seed=8)
    e = covgpu.Engine(N, L, maxslots=nq + 1, maxnull=nq)
    e.set_tree(s.parent, s.left, s.right)
    e.set_alignment(0, s.ax)
    e.set_weights(covgpu.weights_pb(s.ax))
    f = e.learned_features(1.5, nquick=nq).astype(np.float64)
    r = e.rscape(None, None, ["GTp"], nshuffle=nq)[0]
    P = L * (L - 1) // 2
    assert f[47] == pytest.approx(np.log(nq * P), rel=1e-6)
    assert f[60] == pytest.approx(r["mu"], rel=1e-6)
    assert f[61] == pytest.approx(np.log(r["tau"] / r["lambda_"]), rel=1e-5, abs=1e-6)
    assert f[62] == pytest.approx(np.log(r["tau"]), rel=1e-5, abs=1e-6)
    m = r["tau"] / r["lambda_"]
    q = f[50:60]                         # survival 0.5 ... 0.0005: increasing offsets from mu_q
    assert np.all(np.diff(q) >= 0) and q[0] >= f[48] - 3 * f[49]
    # the tail's lower bound mu_q is the 0.0005 quantile's bin, within a bin width
    assert abs(q[-1]) * m <= r["w"] * (1 + 1e-6)
    assert f[63] == pytest.approx((r["h_xmax"] - r["mu"]) / m, rel=1e-5, abs=1e-6)
    assert q[-1] <= f[63] + r["w"] / m
    e.close()


def test_network_forward_and_gradient_match_oracle(covgpu, oracle):
    rng = np.random.default_rng(11)
    net = covgpu.MLP(batch_cap=128, seed=3)
    p = net.params()
    p[16384:16640] = rng.standard_normal(256) * 0.1        # non-zero biases exercise their gradients
    net.set_params(p)
    xm = rng.standard_normal(64).astype(np.float32)
    xs = (0.5 + rng.random(64)).astype(np.float32)
    ym = np.array([5.0, -1.0, 0.3], np.float32)
    ys = np.array([2.0, 0.7, 0.4], np.float32)
    net.set_norm(xm, xs, ym, ys)
    nrm = np.concatenate([xm, xs, ym, ys]).astype(np.float32)
    X = (xm + xs * rng.standard_normal((100, 64))).astype(np.float32)
    T = (ym + ys * rng.standard_normal((100, 3))).astype(np.float32)
    Y = net.forward(X)
    Yr = oracle.mlp_forward(p, nrm, X)
    assert np.allclose(Y, Yr, rtol=1e-4, atol=1e-4 * np.abs(Yr).max()), np.abs(Y - Yr).max()
    loss, g = net.grad(X, T)
    lr, gr = oracle.mlp_grad(p, nrm, X, T)
    assert loss == pytest.approx(lr, rel=1e-5)
    # FP32 activations and accumulation against FP64: relative error of the
    # whole gradient and of each layer's block
    assert np.linalg.norm(g - gr) <= 1e-4 * np.linalg.norm(gr)
    for a, b in ((0, 16384), (16384, 16640), (16640, 82176), (82432, 147968), (148224, 148992), (148992, 148995)):
        assert np.linalg.norm(g[a:b] - gr[a:b]) <= 2e-4 * np.linalg.norm(gr[a:b]) + 1e-9, (a, b)
    net.close()


def test_ensemble_forward_is_the_members_mean(covgpu, oracle):
    """covgpu_mlp_set_members: the forward pass averages the members'
    outputs (the oracle's FP64 network per member, then the mean); training
    parameters are untouched, and clearing the members restores them."""
    rng = np.random.default_rng(12)
    net = covgpu.MLP(batch_cap=64, seed=5)
    xm = rng.standard_normal(64).astype(np.float32)
    xs = (0.5 + rng.random(64)).astype(np.float32)
    ym = np.array([3.0, -0.5, 0.2], np.float32)
    ys = np.array([1.5, 0.6, 0.3], np.float32)
    net.set_norm(xm, xs, ym, ys)
    nrm = np.concatenate([xm, xs, ym, ys]).astype(np.float32)
    X = (xm + xs * rng.standard_normal((150, 64))).astype(np.float32)   # 150 rows: three batches of 64
    single = net.forward(X)
    p0 = net.params()
    members = []
    for k in range(3):
        m = covgpu.MLP(batch_cap=8, seed=20 + k)
        members.append(m.params())
        m.close()
    net.set_members(members)
    Y = net.forward(X)
    Yr = np.mean([oracle.mlp_forward(p, nrm, X) for p in members], axis=0)
    assert np.allclose(Y, Yr, rtol=1e-4, atol=1e-4 * np.abs(Yr).max()), np.abs(Y - Yr).max()
    assert np.array_equal(net.params(), p0)
    with pytest.raises(RuntimeError):
        net.set_members(np.zeros((17, covgpu.NPARAM), np.float32))
    net.set_members([])
    assert np.array_equal(net.forward(X), single)
    net.close()


def test_training_is_reproducible_and_fits(covgpu):
    rng = np.random.default_rng(4)
    X = rng.standard_normal((2048, 64)).astype(np.float32)
    W = rng.standard_normal((64, 3)).astype(np.float32) / 8
    T = np.tanh(X @ W) * 2 + 0.1 * (X[:, :3] ** 2)
    T = T.astype(np.float32)
    runs = []
    for _ in range(2):
        net = covgpu.MLP(batch_cap=256, seed=9)
        net.set_norm(X.mean(0), X.std(0), T.mean(0), T.std(0))
        hist = net.train(X, T, 40, batch=256, lr=2e-3, wd=1e-4, seed=5)
        runs.append((hist, net.params(), net.forward(X[:64])))
        net.close()
    (h1, p1, y1), (h2, p2, y2) = runs
    assert np.array_equal(p1, p2) and np.array_equal(h1, h2)      # fixed summation order
    assert h1[-1] < 0.1 * h1[0]
    assert np.sqrt(np.mean((y1 - T[:64]) ** 2)) < 0.3 * T.std()


def _gamma_sf(tau, x):
    from scipy.special import gammaincc
    return gammaincc(tau, x)


def test_learned_evalues_follow_the_predicted_tail(covgpu):
    """A network whose output is a fixed tail: every E-value must equal
    Nt * pmass * Q(tau, lambda (u - mu)) at the bin bound the full path uses."""
    pytest.importorskip("scipy")
    N, L = 200, 120
    s = covgpu.Synth(N, L, 1.5, 30, 3, 10, 10, 0.08, seed=21)
    e = covgpu.Engine(N, L, maxslots=21, maxnull=20)
    e.set_tree(s.parent, s.left, s.right)
    w = covgpu.weights_pb(s.ax)
    full = e.rscape(s.ax, w, ["GTp"], nshuffle=20)[0]
    mu, tau, lam = full["mu"], full["tau"], full["lambda_"]
    net = covgpu.MLP(batch_cap=8)
    net.set_params(np.zeros(covgpu.NPARAM, np.float32))
    # a constant network whose correction turns the quick nulls' tail into the full fit's
    f = e.learned_features(1.5, nquick=4).astype(np.float64)
    mq, lmq, ltq = f[60], f[61], f[62]
    target = np.array([(mu - mq) / math.exp(lmq), math.log(tau / lam) - lmq, math.log(tau) - ltq], np.float32)
    net.set_norm(np.zeros(64, np.float32), np.ones(64, np.float32), target, np.ones(3, np.float32))
    r, used = e.rscape_learned(None, None, net, 1.5, "GTp", nquick=4, thresh=1e9)
    assert used and r["nshuffle"] == 4 and r["w"] == full["w"]
    assert r["mu"] == pytest.approx(mu, rel=1e-5) and r["tau"] == pytest.approx(tau, rel=1e-5)
    assert r["lambda_"] == pytest.approx(lam, rel=1e-5)
    mu_f, tau_f, lam_f = r["mu"], r["tau"], r["lambda_"]
    Nt = L * (L - 1) / 2
    bmin, wd = -10.0, r["w"]
    assert r["nhit"] == Nt
    worst = 0.0
    for (i, j, sc, E, pv) in r["hits"]:
        b = math.ceil((sc - bmin) / wd - 1)
        u = bmin + (b + 2) * wd
        sf = 1.0 if u <= mu_f else _gamma_sf(tau_f, lam_f * (u - mu_f))
        ref = Nt * 0.0005 * sf
        if ref > 0:
            worst = max(worst, abs(E - ref) / ref)
    assert worst < 1e-7, worst
    # E < 0.05 pairs of the learned path with the full fit's own tail agree
    # with the full path's pairs
    r2, _ = e.rscape_learned(None, None, net, 1.5, "GTp", nquick=4)
    got = {(i, j) for (i, j, *_x) in r2["hits"]}
    exp = {(i, j) for (i, j, *_x) in full["hits"]}
    assert len(got ^ exp) <= max(1, len(exp) // 10)
    net.close()
    e.close()


def test_out_of_range_falls_back_to_simulation(covgpu):
    N, L = 80, 60
    s = covgpu.Synth(N, L, 1.5, 10, 2, 5, 5, 0.08, seed=5)
    e = covgpu.Engine(N, L, maxslots=21, maxnull=20)
    e.set_tree(s.parent, s.left, s.right)
    w = covgpu.weights_pb(s.ax)
    net = covgpu.MLP(batch_cap=8)
    z = np.zeros(64, np.float32)
    # a training range no alignment reaches: log N in [100, 101]
    lo = np.full(64, -1e9, np.float32); hi = np.full(64, 1e9, np.float32)
    lo[0], hi[0] = 100.0, 101.0
    net.set_norm(z, np.ones(64, np.float32), np.zeros(3, np.float32), np.ones(3, np.float32), lo, hi)
    r, used = e.rscape_learned(s.ax, w, net, 1.5, "GTp", nquick=2, nshuffle=20)
    full = e.rscape(None, None, ["GTp"], nshuffle=20)[0]
    assert not used and r["nshuffle"] == 20
    assert r["mu"] == full["mu"] and r["nhit"] == full["nhit"]
    assert not net.in_range(e.learned_features(1.5, nquick=2))
    net.close()
    e.close()


def test_shipped_network_on_held_out_families(covgpu):
    """The shipped network on families it was not trained on (seeds outside
    its training and evaluation ranges): it runs on the quick nulls, and its
    E-values stay near the 200-null ones."""
    import importlib.util
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("learned_null", os.path.join(root, "r-scape_gb300",
                                                                                "learned_null.py"))
    ln = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ln)
    net = ln.load(os.path.join(root, "r-scape_gb300", "learned_null_gtp.npz"))
    nq = int(np.load(os.path.join(root, "r-scape_gb300", "learned_null_gtp.npz"))["nquick"])
    rows = ln.evaluate(net, 300001, 16, 200, nquick=nq, few=0)
    s = ln.summarize(rows, 200)
    net.close()
    assert s["used_net"] >= 14 and s["null_reduction"] >= 5
    assert s["net_finite_frac"] == 1.0
    assert s["net_median_rel_E_error"] < 0.35


def test_network_beats_its_quick_nulls_own_fit(covgpu):
    """What the trained network gains over the method without it: on 40
    held-out families (seeds outside the training and evaluation ranges),
    the E-values from the quick nulls plus the network against those from
    the same quick nulls' own tail fit, both judged by the 200-null fit.
    The network must have the lower median relative E-value error and win
    in most of the families with a tail."""
    import importlib.util
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("learned_null", os.path.join(root, "r-scape_gb300",
                                                                                "learned_null.py"))
    ln = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ln)
    path = os.path.join(root, "r-scape_gb300", "learned_null_gtp.npz")
    net = ln.load(path)
    nq = int(np.load(path)["nquick"])
    rows = ln.evaluate(net, 310001, 40, 200, nquick=nq, few=0)
    s = ln.summarize(rows, 200)
    net.close()
    print("\nheld-out families: %s" % {k: s[k] for k in ("families_with_tail", "net_median_rel_E_error",
                                                            "quick_median_rel_E_error", "net_better_than_quick",
                                                            "null_reduction")})
    assert s["families_with_tail"] >= 15
    assert s["net_median_rel_E_error"] < s["quick_median_rel_E_error"]
    assert s["net_better_than_quick"] > s["families_with_tail"] / 2
