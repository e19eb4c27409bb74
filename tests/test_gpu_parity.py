"""GPU library vs the CPU oracle on the same inputs (needs a GB300).

Tolerances: pair counts and nseff are compared bit-exactly under unit
weights (float weights are quantised to 33 bits, so their counts are within
1e-9 relative); probabilities within 1e-12; every statistic, raw or
APC/ASC-corrected, within 1e-5 relative on each pair of at least 1e-3 of the
largest magnitude and within 1e-8 of that magnitude below it (parity_tol);
null alignments byte for byte; the E < 0.05 pair set exactly, E-values
within 1e-5 relative.
"""
import numpy as np
import pytest

from parity_tol import stat_close

pytestmark = pytest.mark.gpu


def make(covgpu, N, L, seed, unit=False, tree_kind=1, nbp=None):
    nbp = nbp if nbp is not None else max(0, min(L // 6, 20))
    nh = max(1, nbp // 8) if nbp else 0
    hmin = 1 if nbp else 0
    s = covgpu.Synth(N, L, 1.5, nbp, nh, hmin, max(1, nbp), 0.1, seed=seed, tree_kind=tree_kind)
    w = np.ones(N) if unit else covgpu.weights_pb(s.ax) * np.random.default_rng(seed).uniform(0.7, 1.3, N)
    return s, w


SHAPES = [(50, 40), (97, 70), (200, 130), (33, 64), (5, 100), (64, 33)]


@pytest.mark.parametrize("N,L", SHAPES)
def test_counts_unit_weights_bit_exact(covgpu, oracle, N, L):
    s, w = make(covgpu, N, L, 3, unit=True)
    e = covgpu.Engine(N, L)
    e.set_weights(w)
    e.set_alignment(0, s.ax)
    e.score(["GT"])
    pp, ne, ng, pm, ps = e.get_probs(0, w)
    opp, one, ong, opm, ops = oracle.probs(s.ax, w)
    iu = np.triu_indices(L, 1)
    assert np.array_equal(ne[iu], one[iu])
    assert np.array_equal(ng[iu], ong[iu])
    assert np.allclose(pp[iu], opp[iu], rtol=1e-14, atol=0)
    # pm sums one double-float contribution per partner
    assert np.allclose(pm, opm, rtol=1e-12, atol=1e-15)
    assert np.allclose(ps, ops, rtol=1e-12, atol=1e-15)
    e.close()


STATS = ["CHI", "GT", "MI", "MIr", "MIg", "OMES", "RAF", "RAFS", "CCF"]


@pytest.mark.parametrize("N,L", [(97, 70), (200, 130), (5, 100), (50, 40)])
@pytest.mark.parametrize("unit", [True, False])
@pytest.mark.parametrize("corr", ["", "p", "a"])
def test_statistics(covgpu, oracle, N, L, unit, corr):
    s, w = make(covgpu, N, L, 5, unit=unit)
    e = covgpu.Engine(N, L)
    e.set_weights(w)
    e.set_alignment(0, s.ax)
    for k in range(0, len(STATS), 4):
        types = [t + corr for t in STATS[k:k + 4]]
        mm = e.score(types)
        for q, t in enumerate(types):
            ref, (rmin, rmax) = oracle.cov_calculate(t, s.ax, w)
            got = e.get_cov(0, q)
            iu = np.triu_indices(L, 1)
            ok, rel, small = stat_close(got[iu], ref[iu])
            assert ok, "%s N=%d L=%d unit=%s rel %g small %g" % (t, N, L, unit, rel, small)
            assert np.allclose(got.T[iu], got[iu])
            assert np.allclose(mm[0, q], [rmin, rmax], rtol=1e-5, atol=1e-8 * np.max(np.abs(ref[iu]))), \
                (t, mm[0, q], rmin, rmax)
    e.close()


@pytest.mark.parametrize("cls", [0, 1, 2])
def test_classes(covgpu, oracle, cls):
    N, L = 120, 90
    s, w = make(covgpu, N, L, 9)
    e = covgpu.Engine(N, L)
    e.set_weights(w)
    e.set_alignment(0, s.ax)
    types = ["GTp"] if cls == 2 else ["GTp", "MIp", "CHIp", "OMES"]
    e.score(types, covclass=cls)
    for q, t in enumerate(types):
        ref, _ = oracle.cov_calculate(t, s.ax, w, covclass=cls)
        got = e.get_cov(0, q)
        iu = np.triu_indices(L, 1)
        ok, rel, small = stat_close(got[iu], ref[iu])
        assert ok, (t, cls, rel, small)
    e.close()


@pytest.mark.parametrize("N,L", [(40, 60), (150, 97), (7, 45)])
def test_null_alignments_identical(covgpu, oracle, N, L):
    s, w = make(covgpu, N, L, 13)
    s.ax[0, :5] = 15    # unknown residues take random Fitch states
    e = covgpu.Engine(N, L, maxslots=4, maxnull=3)
    e.set_weights(w)
    e.set_alignment(0, s.ax)
    e.set_tree(s.parent, s.left, s.right)
    e.make_nulls(42, 0, 3, 1)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    for q in range(3):
        ref = oracle.null_msa(s.ax, T, 42, q)
        got = e.get_alignment(1 + q)
        assert np.array_equal(got, ref), "null %d differs in %d cells" % (q, int((got != ref).sum()))
    e.close()


def test_null_alignments_written_as_stockholm(covgpu, oracle, tmp_path):
    """The null alignments of an E-valued call, written in R-scape's --outnull
    form (one Stockholm record per null), read back as the oracle's nulls."""
    N, L, ns = 90, 70, 4
    s, w = make(covgpu, N, L, 17)
    e = covgpu.Engine(N, L, maxslots=ns + 1, maxnull=ns)
    e.set_tree(s.parent, s.left, s.right)
    e.rscape(s.ax, w, ["GTp"], nshuffle=ns)
    path = str(tmp_path / "nulls.sto")
    e.write_nulls(path, 1, ns)
    e.close()
    recs = covgpu.read_stockholm(path)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    assert [r[0] for r in recs] == ["null%d" % (k + 1) for k in range(ns)]
    for k, (name, names, ax) in enumerate(recs):
        assert np.array_equal(ax, oracle.null_msa(s.ax, T, 42, k)), name


@pytest.mark.parametrize("counter", ["simt", "tensor"])
@pytest.mark.parametrize("N,L,types", [
    (200, 120, ["GTp"]),
    (150, 100, ["GTp", "MIp", "CHIp", "RAFp"]),
    (60, 45, ["MIa"]),
])
def test_rscape_pipeline(covgpu, oracle, N, L, types, counter):
    """The whole path against the oracle: the width w (from the first null's
    score range), the null histogram, the tail fit, the hits and their
    E-values.  Both counting paths count the same 33-bit quantised weights
    exactly, so they give the same scores."""
    s, w = make(covgpu, N, L, 42, nbp=L // 5)
    ns = 8
    e = covgpu.Engine(N, L, maxslots=ns + 1, maxnull=ns)
    e.set_tree(s.parent, s.left, s.right)
    cnt = covgpu.SIMT if counter == "simt" else covgpu.TENSOR
    rtol = 1e-6
    res = e.rscape(s.ax, w, types, nshuffle=ns, counter=cnt)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    for q, t in enumerate(types):
        ref = oracle.rscape(s.ax, w, T, covtype=t, nshuffle=ns)
        g = res[q]
        assert g["status"] == 0
        assert abs(g["w"] - ref["w"]) <= rtol * abs(ref["w"])
        for k in ("h_nb", "h_imin", "h_imax", "h_cmin", "h_n", "h_Nc", "h_No"):
            assert g[k] == ref[k], (t, k, g[k], ref[k])
        assert abs(g["mu"] - ref["mu"]) <= rtol * (abs(ref["mu"]) + 10.0)
        assert abs(g["lambda_"] - ref["lambda_"]) <= 100 * rtol * abs(ref["lambda_"])
        assert abs(g["tau"] - ref["tau"]) <= 100 * rtol * max(1e-12, abs(ref["tau"]))
        gh = {(i, j): (sc, E) for (i, j, sc, E, p) in g["hits"]}
        rh = {(i, j): (sc, E) for (i, j, sc, E, p) in ref["hits"]}
        assert set(gh) == set(rh), (t, sorted(set(gh) ^ set(rh))[:10])
        for k in rh:
            assert abs(gh[k][1] - rh[k][1]) <= 100 * rtol * rh[k][1] + 1e-300, (t, k, gh[k], rh[k])
    e.close()


@pytest.mark.parametrize("counter", ["simt", "tensor"])
@pytest.mark.parametrize("types", [["GTp"], ["MIp", "CHIp"]])
def test_rscape_pipeline_exponential_tail(covgpu, oracle, counter, types):
    """R-scape's --expo path (cov_NullFitExponential, src/covariation.c:1914-1941):
    the null tail fitted by the binned exponential ML fit instead of the
    gamma; the width, histogram, fit, hits and E-values against the
    oracle's fit_exp."""
    N, L, ns = 180, 110, 8
    s, w = make(covgpu, N, L, 31, nbp=L // 5)
    e = covgpu.Engine(N, L, maxslots=ns + 1, maxnull=ns)
    e.set_tree(s.parent, s.left, s.right)
    cnt = covgpu.SIMT if counter == "simt" else covgpu.TENSOR
    res = e.rscape(s.ax, w, types, nshuffle=ns, counter=cnt, doexpfit=1, thresh=10.0)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    for q, t in enumerate(types):
        ref = oracle.rscape(s.ax, w, T, covtype=t, nshuffle=ns, doexpfit=1, thresh=10.0)
        g = res[q]
        assert g["status"] == 0
        assert abs(g["w"] - ref["w"]) <= 1e-6 * abs(ref["w"])
        for k in ("h_nb", "h_imin", "h_imax", "h_cmin", "h_n", "h_Nc", "h_No"):
            assert g[k] == ref[k], (t, k, g[k], ref[k])
        assert abs(g["mu"] - ref["mu"]) <= 1e-6 * (abs(ref["mu"]) + 10.0)
        assert abs(g["lambda_"] - ref["lambda_"]) <= 1e-6 * abs(ref["lambda_"]), (t, g["lambda_"], ref["lambda_"])
        gh = {(i, j): E for (i, j, sc, E, p) in g["hits"]}
        rh = {(i, j): E for (i, j, sc, E, p) in ref["hits"]}
        assert set(gh) == set(rh) and len(rh) > 0, (t, sorted(set(gh) ^ set(rh))[:10])
        for k in rh:
            assert abs(gh[k] - rh[k]) <= 1e-5 * rh[k] + 1e-300, (t, k, gh[k], rh[k])
    e.close()


def test_rscape_pipeline_fine_bins(covgpu, oracle):
    """A histogram width of 0.002 puts the null scores over ~10^4 bins, so the
    histogram kernel runs with its widest shared-memory window (four groups of
    256 threads per CTA, one CTA per SM); the histogram, the fit and the hits
    must still match the oracle."""
    N, L, ns = 200, 120, 8
    s, w = make(covgpu, N, L, 42, nbp=24)
    e = covgpu.Engine(N, L, maxslots=ns + 1, maxnull=ns)
    e.set_tree(s.parent, s.left, s.right)
    res = e.rscape(s.ax, w, ["GTp", "CHIp"], nshuffle=ns, counter=covgpu.TENSOR, w0=0.002)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    for q, t in enumerate(["GTp", "CHIp"]):
        ref = oracle.rscape(s.ax, w, T, covtype=t, nshuffle=ns, w0=0.002)
        g = res[q]
        assert g["status"] == 0
        # the bins between the smallest and the largest null score all lie in
        # the shared-memory window: more than 14,000 of them is the wide launch
        span = (g["h_xmax"] - g["h_xmin"]) / g["w"]
        assert span > 14000, (t, span)
        for k in ("h_nb", "h_imin", "h_imax", "h_cmin", "h_n", "h_Nc", "h_No"):
            assert g[k] == ref[k], (t, k, g[k], ref[k])
        assert abs(g["mu"] - ref["mu"]) <= 1e-6 * (abs(ref["mu"]) + 10.0)
        assert abs(g["lambda_"] - ref["lambda_"]) <= 1e-4 * abs(ref["lambda_"])
        gh = {(i, j): E for (i, j, sc, E, p) in g["hits"]}
        rh = {(i, j): E for (i, j, sc, E, p) in ref["hits"]}
        assert set(gh) == set(rh)
        for k in rh:
            assert abs(gh[k] - rh[k]) <= 1e-4 * rh[k] + 1e-300
    e.close()


def test_one_sequence(covgpu):
    s, w = make(covgpu, 2, 40, 1)
    e = covgpu.Engine(1, 40, maxslots=2, maxnull=1)
    r = e.rscape(s.ax[:1], np.ones(1), ["GTp"])
    assert r[0]["status"] == 2 and r[0]["nhit"] == 0
    e.close()


def test_constant_alignment(covgpu):
    N, L = 30, 40
    ax = np.zeros((N, L), dtype=np.uint8)
    s, _ = make(covgpu, N, L, 2)
    e = covgpu.Engine(N, L, maxslots=6, maxnull=5)
    e.set_tree(s.parent, s.left, s.right)
    r = e.rscape(ax, np.ones(N), ["GTp"], nshuffle=5)
    assert r[0]["status"] == 1 and r[0]["nhit"] == 0
    e.close()


def test_bad_inputs_rejected(covgpu):
    e = covgpu.Engine(10, 20)
    with pytest.raises(RuntimeError):
        e.set_alignment(0, np.full((10, 20), 99, dtype=np.uint8))
    with pytest.raises(RuntimeError):
        w = np.ones(10)
        w[3] = -1.0
        e.set_weights(w)
    with pytest.raises(RuntimeError):
        e.set_tree(np.zeros(9, np.int32), np.zeros(9, np.int32), np.zeros(9, np.int32))
    e.close()


# ---------------------------------------------------------------------------
# tensor-core counting (tcgen05): counts exact for the quantised weights
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("N,L", [(64, 40), (97, 70), (200, 130), (300, 257)])
@pytest.mark.parametrize("unit", [True, False])
def test_tensor_counts(covgpu, oracle, N, L, unit):
    s, w = make(covgpu, N, L, 17, unit=unit)
    e = covgpu.Engine(N, L)
    e.set_weights(w)
    e.set_alignment(0, s.ax)
    e.score(["GT"], counter=covgpu.TENSOR)
    pp, ne, ng, pm, ps = e.get_probs(0, w)
    opp, one, ong, opm, ops = oracle.probs(s.ax, w)
    iu = np.triu_indices(L, 1)
    if unit:
        assert np.array_equal(ne[iu], one[iu])
        assert np.allclose(pp[iu], opp[iu], rtol=1e-14, atol=0)
    else:
        # weights quantised to 33 bits, counts exact for them (double-float)
        assert np.allclose(ne[iu], one[iu], rtol=1e-9, atol=0)
        assert np.allclose(pp[iu], opp[iu], rtol=1e-9, atol=1e-15)
    assert np.allclose(pm, opm, rtol=1e-9, atol=1e-15)
    e.close()


@pytest.mark.parametrize("N,L", [(97, 70), (200, 130)])
def test_tensor_statistics(covgpu, oracle, N, L):
    s, w = make(covgpu, N, L, 23)
    e = covgpu.Engine(N, L)
    e.set_weights(w)
    e.set_alignment(0, s.ax)
    types = ["GTp", "MIp", "CHIp", "RAFp"]
    e.score(types, counter=covgpu.TENSOR)
    iu = np.triu_indices(L, 1)
    for q, t in enumerate(types):
        ref, _ = oracle.cov_calculate(t, s.ax, w)
        got = e.get_cov(0, q)
        ok, rel, small = stat_close(got[iu], ref[iu])
        assert ok, (t, rel, small)
    e.close()


def test_tensor_pipeline_same_pairs(covgpu, oracle):
    N, L, ns = 200, 120, 8
    s, w = make(covgpu, N, L, 42, nbp=24)
    e = covgpu.Engine(N, L, maxslots=ns + 1, maxnull=ns)
    e.set_tree(s.parent, s.left, s.right)
    simt = e.rscape(s.ax, w, ["GTp"], nshuffle=ns, counter=covgpu.SIMT)[0]
    tens = e.rscape(s.ax, w, ["GTp"], nshuffle=ns, counter=covgpu.TENSOR)[0]
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    ref = oracle.rscape(s.ax, w, T, covtype="GTp", nshuffle=ns)
    exp = sorted((i, j) for (i, j, sc, E, p) in ref["hits"])
    assert sorted((i, j) for (i, j, sc, E, p) in tens["hits"]) == exp
    assert sorted((i, j) for (i, j, sc, E, p) in simt["hits"]) == exp
    e.close()


@pytest.mark.parametrize("seed", [2, 42])
@pytest.mark.parametrize("counter", ["simt", "tensor"])
def test_small_rna_workload(covgpu, oracle, counter, seed):
    """The reference-scale CPU workload end to end: N=100 x L=120, coalescent
    tree of length 1.5, three helices of 10 base pairs, 8% gaps in runs of
    mean 3, position-based FP64 weights, GTp with APC, 20 null alignments.
    The pairs with E < 10 and their E-values are the oracle's (so is the
    E < 0.05 list among them, which this recipe keeps short)."""
    N, L, ns = 100, 120, 20
    s = covgpu.Synth(N, L, 1.5, 30, 3, 10, 10, 0.08, gap_mean=3.0, seed=seed, tree_kind=0)
    assert covgpu.gapfilter(s.ax, None, 0.75).all()
    w = covgpu.weights_pb(s.ax)
    e = covgpu.Engine(N, L, maxslots=ns + 1, maxnull=ns)
    e.set_tree(s.parent, s.left, s.right)
    g = e.rscape(s.ax, w, ["GTp"], thresh=10.0, counter=covgpu.TENSOR if counter == "tensor" else covgpu.SIMT)[0]
    e.close()
    assert g["nshuffle"] == ns          # R-scape's rule gives 20 nulls at this size
    ref = oracle.rscape(s.ax, w, oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd), covtype="GTp",
                        nshuffle=ns, thresh=10.0)
    gh = {(i, j): E for (i, j, sc, E, p) in g["hits"]}
    rh = {(i, j): E for (i, j, sc, E, p) in ref["hits"]}
    assert set(gh) == set(rh) and len(rh) > 0
    for k in rh:
        assert abs(gh[k] - rh[k]) <= 1e-3 * rh[k]
    assert {k for k in gh if gh[k] < 0.05} == {k for k in rh if rh[k] < 0.05}


@pytest.mark.parametrize("variant", ["two_set", "structured", "two_set_structured", "wc_two_set", "all_hits"])
def test_rscape_two_set_and_structured(covgpu, oracle, variant):
    """covgpu_rscape with a structure: the two-set test (R-scape -s: Nb tests
    for the structure's base pairs, P - Nb for the others) and --structured
    (expBP tests for the first hits) against the oracle: numbers of tests,
    both thresholds, the hits and their E-values.  Contacts listed twice
    with different types, and one with i > j, follow the reference's
    matching rules."""
    N, L, ns = 200, 120, 8
    s, w = make(covgpu, N, L, 42, nbp=L // 5)
    bps = [(i, int(s.ct[i])) for i in range(L) if s.ct[i] > i]
    contacts = [(bps[0][0] + 1, bps[0][1] + 1, 5)] + [(i + 1, j + 1, oracle.WWc) for i, j in bps]
    extra = (2, 9) if (1, 8) not in bps else (3, 11)
    contacts += [(extra[0], extra[1], oracle.STACKED), (extra[0], extra[1], oracle.WWc), (40, 12, oracle.WWc)]
    sample = {"two_set": 1, "structured": 3, "two_set_structured": 1, "wc_two_set": 2, "all_hits": 1}[variant]
    expBP = 4.5 if "structured" in variant else (3.0 if variant == "all_hits" else -1.0)
    thresh = 2000.0 if variant == "all_hits" else 0.05
    e = covgpu.Engine(N, L, maxslots=ns + 1, maxnull=ns)
    e.set_tree(s.parent, s.left, s.right)
    kw = dict(nshuffle=ns, samplesize=sample, contacts=contacts, expBP=expBP, thresh=thresh)
    g = e.rscape(s.ax, w, ["GTp"], counter=covgpu.TENSOR, hitcap=1 << 16, **kw)[0]
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    ref = oracle.rscape(s.ax, w, T, covtype="GTp", **kw)
    assert g["Nt"] == ref["Nt"] and g["Nb"] == ref["Nb"]
    if sample != 3:
        assert g["Nb"] > 0
    for k in ("sc_thresh", "sc_nbp"):
        assert abs(g[k] - ref[k]) <= 1e-5 * abs(ref[k]) + 1e-9, (k, g[k], ref[k])
    gh = {(i, j): E for (i, j, sc, E, p) in g["hits"]}
    rh = {(i, j): E for (i, j, sc, E, p) in ref["hits"]}
    assert g["nhit"] == ref["nhit"]
    assert set(gh) == set(rh), sorted(set(gh) ^ set(rh))[:10]
    for k, E in rh.items():
        assert abs(gh[k] - E) <= 1e-4 * E + 1e-300, (k, gh[k], E)
    e.close()


def test_structure_only_in_the_single_alignment_path(covgpu):
    """A structure belongs to one alignment: the family batch and the learned
    null refuse the two-set test and --structured."""
    N, L = 60, 50
    s, w = make(covgpu, N, L, 3)
    fam = dict(ax=s.ax, wgt=w, parent=s.parent, left=s.left, right=s.right)
    b = covgpu.Batch(mem_gb=1.0)
    with pytest.raises(RuntimeError):
        b.rscape([fam], ["GTp"], samplesize=1, contacts=[(1, 10, 0)])
    with pytest.raises(RuntimeError):
        b.rscape([fam], ["GTp"], expBP=5.0)
    b.close()
    e = covgpu.Engine(N, L, maxslots=5, maxnull=4)
    e.set_tree(s.parent, s.left, s.right)
    net = covgpu.MLP(batch_cap=8)
    with pytest.raises(RuntimeError):
        e.rscape_learned(s.ax, w, net, 1.0, "GTp", nquick=4, expBP=5.0)
    net.close()
    e.close()
