"""CPU oracle pinned against the reference's published outputs and against
published known-answer vectors (no GPU)."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def arisong(O):
    d = np.load(os.path.join(HERE, "golden", "arisong.npz"))
    ax = d["ax"]
    use = O.gapfilter(ax, None, 0.75)
    f = ax[:, use].copy()
    f[(f > 4) & (f < 15)] = 15
    f[f > 15] = 4
    return ax, f, np.nonzero(use)[0]


def test_philox_known_answers(oracle):
    # Random123 known-answer vectors for philox4x32-10
    assert oracle.philox([0, 0], [0, 0, 0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle.philox([0xFFFFFFFF] * 2, [0xFFFFFFFF] * 4) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]


def test_arisong_gap_filter(oracle):
    gold = json.load(open(os.path.join(HERE, "golden", "arisong_gtp.json")))
    ax, f, cols = arisong(oracle)
    assert ax.shape == (gold["nseq"], gold["alen"])
    assert f.shape[1] == gold["alen_filtered"]


def test_arisong_gtp_scores(oracle):
    """GTp + APC on the gap-filtered Arisong alignment with GSC weights
    reproduces the tutorial's table (documentation/tutorial.tex:186-212).
    The weights are a restatement of Easel's GSC, so the pin is 0.06 absolute
    on scores of 45-122 (10 of the 11 pairs agree to < 4e-3)."""
    gold = json.load(open(os.path.join(HERE, "golden", "arisong_gtp.json")))
    ax, f, cols = arisong(oracle)
    w = oracle.weights_gsc(f)
    assert abs(w.sum() - f.shape[0]) < 1e-9
    COV, (mn, mx) = oracle.cov_calculate("GTp", f, w)
    assert abs(mx - 121.65824) < 0.01
    errs = []
    for r in gold["pairs"]:
        i = int(np.nonzero(cols == r["left"] - 1)[0][0])
        j = int(np.nonzero(cols == r["right"] - 1)[0][0])
        errs.append(abs(COV[i, j] - r["score"]))
    errs = np.array(errs)
    assert errs.max() < 0.06
    assert np.sum(errs < 4e-3) >= 10
    # the table lists the base pairs by decreasing score; ours keep that order
    sc = []
    for r in gold["pairs"]:
        i = int(np.nonzero(cols == r["left"] - 1)[0][0])
        j = int(np.nonzero(cols == r["right"] - 1)[0][0])
        sc.append(COV[i, j])
    assert all(sc[k] > sc[k + 1] for k in range(len(sc) - 1))


def test_probs_normalised(oracle):
    ax, f, cols = arisong(oracle)
    w = oracle.weights_gsc(f)
    pp, ne, ng, pm, ps = oracle.probs(f, w)
    L = f.shape[1]
    iu = np.triu_indices(L, 1)
    assert np.allclose(pp[iu].sum(-1), 1.0, atol=1e-12)
    assert np.allclose(pm.sum(-1), 1.0, atol=1e-12)
    assert np.allclose(ps.sum(-1), 1.0, atol=1e-12)
    assert np.allclose(ne[iu] + ng[iu], w.sum(), atol=1e-9)
    # pp[j][i] is the transpose of pp[i][j]
    assert np.allclose(pp[3, 7].reshape(4, 4), pp[7, 3].reshape(4, 4).T)


def _direct_raf(ax, allow):
    """RAF from its O(N^2) definition, src/correlators.c:897-925."""
    N, L = ax.shape
    A = allow.reshape(4, 4)
    out = np.zeros((L, L))
    for i in range(L - 1):
        for j in range(i + 1, L):
            ok = np.array([(a < 4 and b < 4 and A[a, b] > 0) for a, b in zip(ax[:, i], ax[:, j])])
            c = 0.0
            for s1 in range(N):
                for s2 in range(s1 + 1, N):
                    if ok[s1] and ok[s2]:
                        d = int(ax[s1, i] != ax[s2, i]) + int(ax[s1, j] != ax[s2, j])
                        c += d
            q = (N - ok.sum()) / N
            out[i, j] = 2 * c / (N * (N - 1)) - q
    return out


def test_raf_matches_definition(oracle):
    rng = np.random.default_rng(3)
    ax = rng.integers(0, 5, size=(9, 7)).astype(np.uint8)
    COV, _ = oracle.cov_calculate("RAF", ax, np.ones(9))
    ref = _direct_raf(ax, oracle.default_allow())
    iu = np.triu_indices(7, 1)
    assert np.allclose(COV[iu], ref[iu], atol=1e-12)


def test_apc_definition(oracle):
    rng = np.random.default_rng(5)
    ax = rng.integers(0, 5, size=(30, 12)).astype(np.uint8)
    w = rng.uniform(0.5, 1.5, 30)
    C, _ = oracle.cov_calculate("MI", ax, w)
    P, _ = oracle.cov_calculate("MIp", ax, w)
    L = 12
    off = ~np.eye(L, dtype=bool)
    colx = np.where(off, C, 0).sum(1) / (L - 1)
    avg = C[np.triu_indices(L, 1)].sum() * 2 / (L * (L - 1))
    ref = C - np.outer(colx, colx) / avg
    assert np.allclose(P[off], ref[off], atol=1e-12)


def test_null_preserves_composition(oracle, covgpu):
    """A null alignment keeps the number of sequences and columns, holds only
    canonical codes and gaps, is the same for the same (seed, null index) and
    differs between null indices."""
    s = covgpu.Synth(40, 60, 1.0, 10, 1, 10, 10, 0.1, seed=7)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    nm = oracle.null_msa(s.ax, T, 42, 3)
    assert nm.shape == s.ax.shape
    assert set(np.unique(nm)) <= {0, 1, 2, 3, 4}
    nm2 = oracle.null_msa(s.ax, T, 42, 3)
    assert np.array_equal(nm, nm2)
    nm3 = oracle.null_msa(s.ax, T, 42, 4)
    assert not np.array_equal(nm, nm3)


def test_feistel_is_permutation(oracle):
    for L in (1, 2, 3, 17, 64, 100, 1000):
        rk = [0x12345678, 0x9ABCDEF0, 7, 11, 13, 17]
        p = [oracle.feistel_perm(t, L, rk) for t in range(L)]
        assert sorted(p) == list(range(L))


def test_rscape_pipeline_small(oracle, covgpu):
    s = covgpu.Synth(200, 120, 1.5, 30, 3, 10, 10, 0.08, seed=42, tree_kind=1)
    w = oracle.weights_pb(s.ax)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    r = oracle.rscape(s.ax, w, T, covtype="GTp", nshuffle=5)
    assert r["nshuffle"] == 5
    assert r["fit_ok"] == 1
    assert r["h_n"] == 5 * 120 * 119 // 2
    assert len(r["hits"]) >= 10
    assert r["null_obs"].sum() == r["h_Nc"]
    # planted pairs dominate the hit list
    ct = s.ct
    planted = sum(1 for (i, j, sc, E, p) in r["hits"] if ct[i] == j)
    assert planted >= max(1, len(r["hits"]) // 2)


def test_empirical_pvalues_follow_the_bin_walk(oracle, covgpu):
    """Below the fitted tail a pair's p-value is the null mass in the score's
    bin and above (cov2evalue, src/covariation.c:2369-2400: the loop over the
    bins imax .. icov).  The oracle takes that mass from a table of suffix
    sums; here every pair of a small alignment (thresh > 1000 lists them all)
    is checked against the loop itself, bit for bit."""
    import math
    s = covgpu.Synth(150, 100, 1.5, 25, 3, 8, 9, 0.08, seed=11, tree_kind=1)
    w = oracle.weights_pb(s.ax)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    r = oracle.rscape(s.ax, w, T, covtype="GTp", nshuffle=8, thresh=2000.0)
    obs = [int(x) for x in r["null_obs"]]
    Nc = float(r["h_Nc"])
    have_sf = r["fit_ok"] == 1 and math.isfinite(r["lambda_"])
    assert len(r["hits"]) == 100 * 99 // 2
    walked = 0
    for (i, j, sc, E, p) in r["hits"]:
        if have_sf and sc >= r["h_phi"]:
            continue
        if sc >= r["h_xmax"]:
            want = 1.0 / Nc
        else:
            icov = int(math.ceil((sc - r["h_bmin"]) / r["h_w"] - 1.0))
            assert icov <= r["h_imax"]
            icov = max(icov, r["h_imin"])
            if icov >= r["h_imax"] - 1:
                want = 1.0 / Nc
            else:
                c = 0
                for b in range(r["h_imax"], icov - 1, -1):
                    c += obs[b]
                want = float(c) * 1.0 / Nc
                walked += 1
        assert p == want, (i, j, sc, p, want)
    assert walked > 1000


def test_c16_statistics_match_definitions(oracle):
    """CHI, OMES, GT, MI, MIr and MIg of the C16 class from the oracle's own
    pair probabilities, marginals and nseff, written out cell by cell
    (src/correlators.c: CHI :92-122, OMES :224-252, GT :359-390, MI :536-561,
    MIr :659-690, MIg :792-822)."""
    rng = np.random.default_rng(11)
    N, L = 40, 9
    ax = rng.integers(0, 5, size=(N, L)).astype(np.uint8)
    w = rng.uniform(0.5, 1.5, N)
    pp, ne, ng, pm, _ = oracle.probs(ax, w)
    ref = {k: np.zeros((L, L)) for k in ("CHI", "OMES", "GT", "MI", "MIr", "MIg")}
    for i in range(L):
        for j in range(i + 1, L):
            p = pp[i, j].reshape(4, 4)
            q = np.outer(pm[i], pm[j])
            o, e = ne[i, j] * p, ne[i, j] * q
            mi = float(np.sum(p * (np.log(p) - np.log(q))))
            h = float(-np.sum(p * np.log(p)))
            ref["CHI"][i, j] = np.sum((o - e) ** 2 / e)
            ref["OMES"][i, j] = np.sum((o - e) ** 2) / ne[i, j]
            ref["GT"][i, j] = 2.0 * np.sum(o * np.log(o / e))
            ref["MI"][i, j] = mi
            ref["MIr"][i, j] = mi / h if h > 1e-2 else 0.0
            ref["MIg"][i, j] = mi - ng[i, j] / ne[i, j]
    iu = np.triu_indices(L, 1)
    for t, R in ref.items():
        got, _ = oracle.cov_calculate(t, ax, w, covclass=oracle.C16)
        assert np.allclose(got[iu], R[iu], rtol=1e-12, atol=1e-12), t


def test_c2_and_cwc_statistics_match_definitions(oracle):
    """The C2 class (cells merged into allowed and not allowed pairs) and the
    GT CWC form (allowed cells only) from the oracle's pair probabilities
    (src/correlators.c: CHI :137-168, OMES :269-301, GT :426-463 and
    :393-423, MI :575-605, MIr :705-736)."""
    rng = np.random.default_rng(12)
    N, L = 30, 8
    ax = rng.integers(0, 5, size=(N, L)).astype(np.uint8)
    w = rng.uniform(0.5, 1.5, N)
    pp, ne, ng, pm, _ = oracle.probs(ax, w)
    allow = np.asarray(oracle.default_allow()).reshape(4, 4) > 0
    ref = {k: np.zeros((L, L)) for k in ("CHI", "OMES", "GT", "MI", "MIr", "CWC")}
    for i in range(L):
        for j in range(i + 1, L):
            p = pp[i, j].reshape(4, 4)
            q = np.outer(pm[i], pm[j])
            n = ne[i, j]
            pw, pn, qw, qn = p[allow].sum(), p[~allow].sum(), q[allow].sum(), q[~allow].sum()
            o, e = n * np.array([pw, pn]), n * np.array([qw, qn])
            mi = pw * np.log(pw / qw) + pn * np.log(pn / qn)
            h = -(pw * np.log(pw) + pn * np.log(pn))
            ref["CHI"][i, j] = np.sum((o - e) ** 2 / e)
            ref["OMES"][i, j] = np.sum((o - e) ** 2) / n
            ref["GT"][i, j] = 2.0 * np.sum(o * np.log(o / e))
            ref["MI"][i, j] = mi
            ref["MIr"][i, j] = mi / h if h > 1e-2 else 0.0
            oc, ec = n * p[allow], n * q[allow]
            ref["CWC"][i, j] = 2.0 * np.sum(oc * np.log(oc / ec))
    iu = np.triu_indices(L, 1)
    for t in ("CHI", "OMES", "GT", "MI", "MIr"):
        got, _ = oracle.cov_calculate(t, ax, w, covclass=oracle.C2)
        assert np.allclose(got[iu], ref[t][iu], rtol=1e-12, atol=1e-12), t
    got, _ = oracle.cov_calculate("GT", ax, w, covclass=oracle.CWC)
    assert np.allclose(got[iu], ref["CWC"][iu], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("N,L,seed", [(40, 30, 1), (97, 50, 2), (7, 25, 3)])
def test_raf_count_form_equals_the_loop(oracle, N, L, seed):
    """The deep-alignment RAF of the oracle (unit counts of the allowed
    cells) against its restatement of corr_CalculateRAF's O(N^2) loop
    (src/correlators.c:876-933), including gaps and unknown residues."""
    rng = np.random.default_rng(seed)
    ax = rng.integers(0, 5, size=(N, L)).astype(np.uint8)
    ax[rng.random((N, L)) < 0.05] = 15
    allow = oracle.default_allow()
    a, b = np.zeros(L * L), np.zeros(L * L)
    mma, mmb = np.zeros(2), np.zeros(2)
    assert oracle.lib().orc_raf(ax, N, L, allow, a, mma) == 0
    assert oracle.lib().orc_raf_counts(ax, N, L, allow, b, mmb) == 0
    iu = np.triu_indices(L, 1)
    assert np.allclose(a.reshape(L, L)[iu], b.reshape(L, L)[iu], rtol=0, atol=1e-15)
    assert np.allclose(mma, mmb, rtol=0, atol=1e-15)


def _replay_structured(E_one, P, expBP, thresh):
    """cov_CreateHitList's --structured rule (src/covariation.c:850-854) by
    hand, from the one-set E-values (E = p * P): pairs in scan order take
    expBP tests while fewer than expBP hits were listed, then P."""
    L = E_one.shape[0]
    out = np.full_like(E_one, np.inf)
    h = 0
    for i in range(L - 1):
        for j in range(i + 1, L):
            pv = E_one[i, j] / P
            e = pv * expBP if h < expBP else pv * P
            out[i, j] = e
            if e < thresh:
                h += 1
    return out


def test_two_set_test_and_structured(oracle, covgpu):
    """The two-set test (R-scape -s; src/covariation.c:414-457, 490-500,
    828-870): the structure's base pairs form their own set of Nb tests,
    the other pairs Nt = P - Nb; the null histogram does not change.  With
    --structured (expBP) the first hits take expBP tests.  With a PDB map,
    pairs closer than mind are left out of the ranking and of Nt."""
    L, P = 120, 120 * 119 // 2
    s = covgpu.Synth(200, L, 1.5, 30, 3, 10, 10, 0.08, seed=42, tree_kind=1)
    w = oracle.weights_pb(s.ax)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    bps = [(i, int(s.ct[i])) for i in range(L) if s.ct[i] > i]
    # planted pairs as WWc; one extra pair listed first as STACKED, then as
    # WWc: the ranking's any-match rule counts it as a base pair, the hit
    # list's first-match type does not
    extra = (1, 7) if (0, 6) not in bps else (2, 9)
    contacts = [(extra[0], extra[1], oracle.STACKED), (extra[0], extra[1], oracle.WWc)]
    contacts += [(i + 1, j + 1, oracle.WWc) for i, j in bps]
    kw = dict(covtype="GTp", nshuffle=5, want_matrices=True, contacts=contacts)
    one = oracle.rscape(s.ax, w, T, **kw)
    two = oracle.rscape(s.ax, w, T, samplesize=oracle.SAMPLE_BP, **kw)
    assert one["Nt"] == P and one["Nb"] == 0 and one["sc_nbp"] == one["sc_thresh"]
    assert two["Nb"] == len(bps) + 1 and two["Nt"] == P - len(bps) - 1
    assert np.array_equal(one["null_obs"], two["null_obs"])
    assert two["sc_thresh"] < two["sc_nbp"]
    iu = np.triu_indices(L, 1)
    bp = np.zeros((L, L), bool)
    for i, j in bps:
        bp[i, j] = True
    pv = one["Eval"][iu] / P
    mult = np.where(bp[iu], two["Nb"], two["Nt"]).astype(np.float64)
    assert np.allclose(two["Eval"][iu], pv * mult, rtol=1e-14, atol=0)
    nbp = lambda r: sum(1 for (i, j, sc, E, p) in r["hits"] if bp[i, j])
    assert nbp(two) >= nbp(one) and nbp(two) >= 1
    # --structured: expBP tests for the first hits
    for expBP in (3.5, 1e9):
        st = oracle.rscape(s.ax, w, T, expBP=expBP, **kw)
        ref = _replay_structured(one["Eval"], P, expBP, 0.05)
        assert np.allclose(st["Eval"][iu], ref[iu], rtol=1e-14, atol=0)
        assert len(st["hits"]) == int(np.sum(ref[iu] < 0.05))
    # the PDB distance rule: pairs with j - i < 4 are not ranked
    m2p = np.arange(L, dtype=np.int32)
    pdb = oracle.rscape(s.ax, w, T, msa2pdb=m2p, mind=4, **kw)
    assert pdb["Nt"] == P - (3 * L - 6)
    assert pdb["h_n"] == 5 * (P - (3 * L - 6))


@pytest.mark.parametrize("doexpfit", [0, 1])
def test_tail_fit_maximises_the_binned_likelihood(oracle, covgpu, doexpfit):
    """The oracle's tail fit (esl_gam_FitCompleteBinned / esl_exp_FitCompleteBinned
    restated: location at phi, binned maximum likelihood over the tail bins
    cmin .. imax) against scipy's optimiser of the same binned likelihood,
    written here from its definition."""
    sp = pytest.importorskip("scipy.special")
    so = pytest.importorskip("scipy.optimize")
    s = covgpu.Synth(160, 110, 1.5, 25, 3, 8, 9, 0.08, seed=23, tree_kind=1)
    w = oracle.weights_pb(s.ax)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    r = oracle.rscape(s.ax, w, T, covtype="GTp", nshuffle=20, doexpfit=doexpfit)
    assert r["fit_ok"] == 1
    obs = r["null_obs"].astype(np.float64)
    bmin, bw, mu = r["h_bmin"], r["h_w"], r["h_phi"]
    bins = [b for b in range(r["h_cmin"], r["h_imax"] + 1) if obs[b] > 0]
    assert len(bins) >= 5
    lo = np.maximum(bmin + np.array(bins) * bw, mu) - mu
    hi = bmin + (np.array(bins) + 1) * bw - mu
    n = obs[bins]

    def nll(lam, tau):
        p = sp.gammaincc(tau, lam * lo) - sp.gammaincc(tau, lam * hi) if not doexpfit else \
            np.exp(-lam * lo) - np.exp(-lam * hi)
        return -np.sum(n * np.log(np.maximum(p, 1e-300)))

    assert r["mu"] == mu
    if doexpfit:
        best = so.minimize_scalar(lambda t: nll(np.exp(t), 1.0), bracket=(np.log(r["lambda_"]) - 1,
                                                                         np.log(r["lambda_"]) + 1), tol=1e-12)
        assert abs(np.exp(best.x) - r["lambda_"]) <= 1e-5 * r["lambda_"]
    else:
        x0 = [np.log(r["lambda_"]) + 0.3, np.log(r["tau"]) - 0.3]
        best = so.minimize(lambda x: nll(np.exp(x[0]), np.exp(x[1])), x0, method="Nelder-Mead",
                           options={"xatol": 1e-10, "fatol": 1e-12, "maxiter": 20000})
        assert abs(np.exp(best.x[0]) - r["lambda_"]) <= 1e-4 * r["lambda_"]
        assert abs(np.exp(best.x[1]) - r["tau"]) <= 1e-4 * r["tau"]
        assert nll(r["lambda_"], r["tau"]) <= best.fun + 1e-7 * abs(best.fun)


def test_position_based_weights_match_the_definition(oracle):
    """Henikoff & Henikoff 1994 position-based weights (R-scape's choice above
    1,000 sequences, src/R-scape.c:1556): per column, a sequence with residue
    x scores 1 / (number of residue types in the column x sequences with x);
    gaps and non-canonical codes score nothing; weights summed over columns
    and scaled to sum to N."""
    rng = np.random.default_rng(8)
    ax = rng.integers(0, 6, size=(37, 29)).astype(np.uint8)   # 4, 5: gap and a degenerate code
    ax[:, 3] = 4                                               # a column of gaps only
    N, L = ax.shape
    ref = np.zeros(N)
    for c in range(L):
        col = ax[:, c]
        types = [x for x in range(4) if np.any(col == x)]
        for s in range(N):
            if col[s] < 4:
                ref[s] += 1.0 / (len(types) * np.sum(col == col[s]))
    ref *= N / ref.sum()
    assert np.allclose(oracle.weights_pb(ax), ref, rtol=1e-13, atol=0)


def _gsc_by_scipy(ax):
    """Gerstein, Sonnhammer & Chothia 1994 weights on scipy's UPGMA tree:
    distance 1 - identities / min(residues) over the columns where both
    sequences carry a residue; each leaf starts with its branch to its
    parent, and the branch above an internal node is shared among the leaves
    below it in proportion to their weights; scaled to sum to N."""
    from scipy.cluster.hierarchy import linkage
    N = ax.shape[0]
    res = ax < 4
    D = np.zeros((N, N))
    for a in range(N):
        for b in range(a + 1, N):
            m = min(res[a].sum(), res[b].sum())
            ident = np.sum((ax[a] == ax[b]) & res[a] & res[b])
            D[a, b] = D[b, a] = 1.0 - ident / m if m > 0 else 1.0
    Z = linkage(D[np.triu_indices(N, 1)], method="average")
    leaves, height, w = {k: [k] for k in range(N)}, {k: 0.0 for k in range(N)}, np.zeros(N)
    for t, (a, b, d, _) in enumerate(Z):
        a, b, h = int(a), int(b), d / 2.0
        for ch in (a, b):
            bl, lv = h - height[ch], leaves[ch]
            if ch < N:
                w[ch] += bl
            elif w[lv].sum() > 0:
                w[lv] += bl * w[lv] / w[lv].sum()
            else:
                w[lv] += bl / len(lv)
        leaves[N + t], height[N + t] = leaves[a] + leaves[b], h
    return w * N / w.sum()


@pytest.mark.parametrize("seed", [0, 7, 19])
def test_gsc_weights_on_an_independent_upgma(oracle, seed):
    """The oracle's GSC weights (R-scape's choice up to 1,000 sequences,
    src/R-scape.c:1555) against the same rule on scipy's UPGMA."""
    pytest.importorskip("scipy.cluster.hierarchy")
    rng = np.random.default_rng(seed)
    base = rng.integers(0, 4, size=300)
    ax = np.array([np.where(rng.random(300) < rng.uniform(0.05, 0.5), rng.integers(0, 5, 300), base)
                   for _ in range(25)]).astype(np.uint8)
    assert np.allclose(oracle.weights_gsc(ax), _gsc_by_scipy(ax), rtol=1e-12, atol=0)


@pytest.mark.parametrize("fracfit,pmass", [(1.0, 0.0005), (0.3, 0.0005), (1.0, 0.05)])
def test_tail_mass_and_tail_bins_follow_the_rules(oracle, covgpu, fracfit, pmass):
    """cov_histogram_pmass (src/covariation.c:2483-2505: walk the non-empty
    bins down from the top until fracfit of them or pmass of the mass is
    passed) and the tail by mass (the smallest top set of bins holding at
    least that mass; its lowest bin is cmin, its lower bound phi), written
    here from the rules, against the oracle's histogram fields."""
    s = covgpu.Synth(150, 100, 1.5, 25, 3, 8, 9, 0.08, seed=29, tree_kind=1)
    w = oracle.weights_pb(s.ax)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    r = oracle.rscape(s.ax, w, T, covtype="GTp", nshuffle=10, pmass=pmass, fracfit=fracfit)
    obs = [int(x) for x in r["null_obs"]]
    imin, imax, n = r["h_imin"], r["h_imax"], r["h_n"]
    assert sum(obs) == n
    tp = sum(1 for b in range(imin, imax + 1) if obs[b] > 0)
    c, nfit, want = 0, 0, None
    for b in range(imax, imin - 1, -1):
        c += obs[b]
        if obs[b] > 0:
            nfit += 1
            want = c / n
            if nfit / tp >= fracfit or want >= pmass:
                break
    assert r["pmass_used"] == want
    acc = 0
    for b in range(imax, imin - 1, -1):
        acc += obs[b]
        if acc >= want * n:
            break
    assert r["h_cmin"] == max(b, imin)
    assert r["newmass"] == acc / n
    assert r["h_phi"] == r["h_bmin"] + r["h_cmin"] * r["h_w"] or \
        abs(r["h_phi"] - (r["h_bmin"] + r["h_cmin"] * r["h_w"])) <= 1e-12 * abs(r["h_phi"])


def test_histogram_width_from_the_first_null(oracle, covgpu):
    """calculate_width_histo (src/R-scape.c:1281-1371): the bin width is
    min(w0, (maxCOV - max(bmin, minCOV)) / hpts) of the first null's scores,
    0 below tol."""
    s = covgpu.Synth(120, 90, 1.5, 20, 2, 8, 10, 0.08, seed=31, tree_kind=1)
    w = oracle.weights_pb(s.ax)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    for hpts, w0 in ((400, 0.05), (40, 0.05), (400, 1e-4)):
        r = oracle.rscape(s.ax, w, T, covtype="MIp", nshuffle=3, hpts=hpts, w0=w0)
        want = min(w0, (r["null_maxCOV"] - max(-10.0, r["null_minCOV"])) / hpts)
        want = 0.0 if want < 1e-6 else want
        assert r["w"] == want, (hpts, w0, r["w"], want)
