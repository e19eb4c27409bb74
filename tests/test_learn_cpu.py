"""Learned null on the CPU: the oracle's network gradient against finite
differences, the oracle's features against their definitions, and the host
logic of the training driver (family draws, standardisation, E-value
comparison)."""
import importlib.util
import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _learned_null():
    spec = importlib.util.spec_from_file_location("learned_null", os.path.join(ROOT, "r-scape_gb300",
                                                                                "learned_null.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def bf16_round(a):
    """Round-to-nearest-even of float32 values to bfloat16 (as float32)."""
    u = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def bf16_step(x, up):
    """The next bfloat16 value above (up) or below x (x a bfloat16 value)."""
    u = np.array([x], dtype=np.float32).view(np.uint32)[0]
    if (x > 0) == up:
        u = u + 0x10000
    else:
        u = u - 0x10000
    return np.array([u], dtype=np.uint32).view(np.float32)[0]


NRM_ID = np.concatenate([np.zeros(64), np.ones(64), np.zeros(3), np.ones(3)]).astype(np.float32)


def test_oracle_gradient_matches_finite_differences(oracle):
    rng = np.random.default_rng(5)
    p = bf16_round(rng.standard_normal(148995) * 0.08)
    X = rng.standard_normal((6, 64)).astype(np.float32)
    T = rng.standard_normal((6, 3)).astype(np.float32)
    loss, g = oracle.mlp_grad(p, NRM_ID, X, T)
    # biases are FP32 in the network: central differences with a small step
    for k in [16384, 16384 + 77, 82176 + 5, 147968 + 200, 148992, 148994]:
        h = 1e-3
        q = p.copy(); q[k] += h
        lp, _ = oracle.mlp_grad(q, NRM_ID, X, T)
        q = p.copy(); q[k] -= h
        lm, _ = oracle.mlp_grad(q, NRM_ID, X, T)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[k]) <= 2e-3 * max(1e-3, abs(g[k])) + 1e-6, (k, fd, g[k])
    # weights are rounded to BF16: step to the neighbouring BF16 values
    for k in [3, 16383, 16640 + 1000, 82432 + 4321, 148224 + 17, 148224 + 700]:
        up, dn = bf16_step(p[k], True), bf16_step(p[k], False)
        q = p.copy(); q[k] = up
        lp, _ = oracle.mlp_grad(q, NRM_ID, X, T)
        q = p.copy(); q[k] = dn
        lm, _ = oracle.mlp_grad(q, NRM_ID, X, T)
        fd = (lp - lm) / (float(up) - float(dn))
        assert abs(fd - g[k]) <= 2e-2 * max(1e-3, abs(g[k])) + 1e-5, (k, fd, g[k])


def test_oracle_forward_denormalises(oracle):
    rng = np.random.default_rng(2)
    p = np.zeros(148995, np.float32)
    p[148992:] = [0.5, -1.0, 2.0]
    nrm = NRM_ID.copy()
    nrm[128:131] = [1.0, 2.0, 3.0]
    nrm[131:134] = [2.0, 0.5, 0.25]
    Y = oracle.mlp_forward(p, nrm, rng.standard_normal((4, 64)))
    assert np.allclose(Y, np.array([1.0 + 2 * 0.5, 2.0 - 0.5, 3.0 + 0.5])[None, :])


def test_oracle_features_definitions(oracle):
    rng = np.random.default_rng(3)
    N, L = 30, 40
    ax = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
    ax[:, 0] = 2          # a conserved column: entropy 0
    ax[:, 1] = 4          # an all-gap column
    ax[:15, 2] = 0        # two residues in equal numbers: entropy 1 bit
    ax[15:, 2] = 3
    w = np.ones(N)
    f = oracle.features(ax, w, 0.7)
    assert f[0] == pytest.approx(math.log(N)) and f[1] == pytest.approx(math.log(L))
    assert f[2] == pytest.approx(math.log(N))                       # unit weights: Neff = N
    assert f[4] == 0.7 and f[42] == pytest.approx(0.0)
    for q in range(2):
        assert f[5 + 16 * q: 21 + 16 * q].sum() == pytest.approx(1.0)
    assert f[43:47].sum() == pytest.approx(1.0)
    assert np.all(f[47:] == 0.0)                                     # the null-score summary is the engine's
    # column statistics from their definitions
    H, g = [], []
    for c in range(L):
        col = ax[:, c]
        n = np.array([(col == x).sum() for x in range(4)], float)
        r = n.sum()
        p = n[n > 0] / r if r else np.array([])
        H.append(float(-(p * np.log2(p)).sum()) if r else 0.0)
        g.append((N - r) / N)
    assert f[38] == pytest.approx(np.mean(H)) and f[39] == pytest.approx(np.std(H))
    assert f[40] == pytest.approx(np.mean(g)) and f[41] == pytest.approx(np.std(g))
    hH = np.bincount(np.minimum(15, (np.array(H) * 8).astype(int)), minlength=16) / L
    assert np.allclose(f[5:21], hH)
    assert f[5] == pytest.approx(np.mean(np.array(H) < 0.125)) and f[5] >= 1.0 / L
    # N(N-1)/2 = 435 <= 4096: every pair
    ids = []
    for i in range(N):
        for j in range(i + 1, N):
            both = (ax[i] < 4) & (ax[j] < 4)
            ids.append(((ax[i] == ax[j]) & both).sum() / both.sum())
    assert f[3] == pytest.approx(np.mean(ids)) and f[37] == pytest.approx(np.std(ids))
    # identical sequences: identity 1
    f1 = oracle.features(np.tile(ax[:1], (5, 1)), np.ones(5), 0.0)
    assert f1[3] == pytest.approx(1.0) and f1[37] == pytest.approx(0.0)


def test_family_draws_follow_the_ragged_recipe():
    ln = _learned_null()
    fams = [ln.draw_family(s) for s in range(1, 400)]
    N = np.array([f["N"] for f in fams])
    L = np.array([f["L"] for f in fams])
    assert N.min() >= 20 and N.max() <= 2000 and L.min() >= 50 and L.max() <= 1500
    assert all(0.5 <= f["tree_len"] <= 3.0 and 0.1 <= f["bp_frac"] <= 0.35 for f in fams)
    # log-uniform L: the median sits near sqrt(50 * 1500)
    assert 150 < np.median(L) < 400
    for f in fams:   # the planted helices fit (2 nbp + 4 nhelix <= L) and respect hmin <= nbp/nhelix <= hmax
        assert 2 * f["nbp"] + 4 * f["nhelix"] <= f["L"]
        assert f["hmin"] * f["nhelix"] <= f["nbp"] <= f["hmax"] * f["nhelix"]
    assert ln.draw_family(7) == ln.draw_family(7)


def test_tree_depth_and_norm():
    ln = _learned_null()
    # root 0 -> (node 1, leaf 0); node 1 -> (leaf 1, leaf 2)
    parent = np.array([-1, 0]); left = np.array([1, -1]); right = np.array([0, -2])
    ld = np.array([1.0, 0.5]); rd = np.array([2.0, 0.25])
    assert ln.tree_depth(parent, left, right, ld, rd) == pytest.approx((2.0 + 1.5 + 1.25) / 3)
    X = np.random.default_rng(1).standard_normal((50, 64)).astype(np.float32)
    X[:, 5] = 3.0                      # a constant feature keeps a unit scale
    T = np.random.default_rng(2).standard_normal((50, 3)).astype(np.float32)
    xm, xs, ym, ys, lo, hi = ln.norm_of(X, T)
    assert xs[5] == 1.0 and np.all(lo <= X.min(0)) and np.all(hi >= X.max(0))


def test_evalue_errors():
    ln = _learned_null()
    truth = {"hits": [(0, 1, 9.0, 0.01, 0), (0, 2, 8.0, 0.5, 0), (1, 2, 5.0, 2.0, 0)]}
    other = {"hits": [(0, 1, 9.0, 0.011, 0), (0, 3, 1.0, 0.04, 0)]}
    errs, agree, na, nb = ln.evalue_errors(truth, other)
    assert errs[0] == pytest.approx(0.1) and errs[1] == float("inf") and len(errs) == 2
    assert na == 1 and nb == 2 and agree == pytest.approx(0.5)


def test_shipped_network_file(oracle):
    """The trained networks shipped with the package: complete, finite, and
    their training range contains their own mean features; an ensemble file
    holds one parameter row per member (at most 16), each a working network."""
    for name in ("learned_null_gtp.npz", "learned_null_gtp_q10.npz"):
        z = np.load(os.path.join(ROOT, "r-scape_gb300", name))
        P = np.atleast_2d(z["params"])
        assert P.shape[1:] == (148995,) and 1 <= len(P) <= 16 and np.all(np.isfinite(P))
        assert int(z["nquick"]) >= 1
        assert np.all(z["xstd"] > 0) and np.all(z["ystd"] > 0)
        assert np.all(z["xlo"] <= z["xmean"]) and np.all(z["xmean"] <= z["xhi"])
        nrm = np.concatenate([z["xmean"], z["xstd"], z["ymean"], z["ystd"]]).astype(np.float32)
        for p in P:
            y = oracle.mlp_forward(p, nrm, z["xmean"][None, :])
            assert np.all(np.isfinite(y)) and np.all(np.abs(y) < 5)


def test_training_data_conversion(tmp_path):
    """Files without the summary="relative" tag hold the quick-null summary as
    absolute scores and are converted; tagged files are read as they are;
    mixed numbers of quick nulls are refused."""
    ln = _learned_null()
    rng = np.random.default_rng(4)
    X = rng.standard_normal((5, 64)).astype(np.float32)
    X[:, 61] = rng.uniform(-1, 1, 5)             # log m_q
    T = rng.standard_normal((5, 3)).astype(np.float32)
    old, new = tmp_path / "old.npz", tmp_path / "new.npz"
    np.savez(old, X=X, T=T, nquick=10)
    np.savez(new, X=X, T=T, nquick=10, summary="relative")
    Xa, Ta, nq = ln.load_training_data([str(old), str(new)])
    assert nq == 10 and Xa.shape == (10, 64) and np.array_equal(Ta, np.concatenate([T, T]))
    m = np.exp(X[:, 61].astype(np.float64))
    assert np.allclose(Xa[:5, 48], (X[:, 48] - X[:, 60]) / m, rtol=1e-5, atol=1e-6)
    assert np.allclose(Xa[:5, 55], (X[:, 55] - X[:, 60]) / m, rtol=1e-5, atol=1e-6)
    assert np.allclose(Xa[:5, 49], X[:, 49] / m, rtol=1e-5, atol=1e-6)
    assert np.array_equal(Xa[:5, :48], X[:, :48]) and np.array_equal(Xa[:5, 60:63], X[:, 60:63])
    assert np.array_equal(Xa[5:], X)             # tagged: unchanged
    Xb, _, _ = ln.load_training_data([str(new)], absolute_summary=True)
    assert np.array_equal(Xb, Xa[:5])             # forced conversion
    other = tmp_path / "other.npz"
    np.savez(other, X=X, T=T, nquick=4, summary="relative")
    with pytest.raises(ValueError):
        ln.load_training_data([str(new), str(other)])


def test_summarize_counts_only_families_with_a_tail():
    """Medians over the families the network handled that have a pair with
    true E < 1; pair-set agreement over the families where either side finds
    an E < 0.05 pair; the simulation saving from the null counts."""
    ln = _learned_null()
    rows = [
        dict(used_net=True, ntail=3, ntrue=1, sim_nulls=10, net_med=0.1, net_agree=1.0, net_nsig=1,
             quick_med=0.3, quick_agree=0.5, quick_nsig=2),
        dict(used_net=True, ntail=2, ntrue=0, sim_nulls=10, net_med=0.2, net_agree=0.0, net_nsig=0,
             quick_med=0.1, quick_agree=1.0, quick_nsig=1),
        dict(used_net=True, ntail=0, ntrue=0, sim_nulls=10, net_med=float("inf"), net_agree=1.0, net_nsig=0,
             quick_med=float("inf"), quick_agree=1.0, quick_nsig=0),
        dict(used_net=False, ntail=4, ntrue=2, sim_nulls=200),
    ]
    s = ln.summarize(rows, 200)
    assert s["families"] == 4 and s["used_net"] == 3 and s["fallback"] == 1 and s["families_with_tail"] == 2
    assert s["simulated_nulls"] == 230 and s["full_nulls"] == 800
    assert s["null_reduction"] == pytest.approx(800 / 230)
    assert s["net_median_rel_E_error"] == pytest.approx(0.15) and s["quick_median_rel_E_error"] == pytest.approx(0.2)
    assert s["net_better_than_quick"] == 1
    # agreement: rows 0 (true pairs) and 1 (quick finds one; the net none)
    assert s["net_pairset_agreement_mean"] == pytest.approx(1.0)
    assert s["quick_pairset_agreement_mean"] == pytest.approx(0.75)
