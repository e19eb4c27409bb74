"""Full-size parity of the E-valued path against the FP64 oracle (needs a
GB300).

* rRNA scale: N=2,000 x L=3,000 synthetic alignment (tree length 2.0, 900
  planted base pairs in 40 helices of 8-35 pairs, 15% gaps in runs of mean
  3, R-scape's 0.75 gap-column filter, position-based weights), 20 null
  alignments, GTp, MIp, CHIp and RAFp with APC, counted on the tensor cores
  and on SIMT.
* batched nulls: N=500 x L=400 (tree length 1.5, 100 base pairs), 200 null
  alignments, GTp with APC.

Each is run through covgpu_rscape and through the oracle's restatement of
null_rscape (src/R-scape.c:1614-1724: the same Fitch + shuffled-substitution
null alignments, scored, binned, tail-fitted) and cov_CreateHitList
(src/covariation.c:778-1006), the statistics sharing one set of nulls.
Compared: the bin width w, every field of the null histogram, the tail fit,
the input alignment's score range, and the pairs with their E-values at
E < 1000 (hundreds to thousands of pairs at these sizes), E < 10 and
E < 0.05.  The last two sets are short here: the phylogenetic signal of
the coalescent tree keeps most planted pairs' E-values above 0.05.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THRESH = 1000.0


def rrna_workload(covgpu):
    s = covgpu.Synth(2000, 3000, 2.0, 900, 40, 8, 35, 0.15, gap_mean=3.0, seed=42)
    keep = covgpu.gapfilter(s.ax, None, 0.75)
    ax = np.ascontiguousarray(s.ax[:, keep])
    return s, ax, covgpu.weights_pb(ax)


def compare(g, ref, t):
    assert g["status"] == 0
    assert abs(g["w"] - ref["w"]) <= 1e-7 * abs(ref["w"]), (t, g["w"], ref["w"])
    for k in ("h_nb", "h_imin", "h_imax", "h_cmin", "h_n", "h_Nc", "h_No"):
        assert g[k] == ref[k], (t, k, g[k], ref[k])
    assert abs(g["maxCOV"] - ref["maxCOV"]) <= 1e-5 * abs(ref["maxCOV"]), (t, g["maxCOV"], ref["maxCOV"])
    assert abs(g["minCOV"] - ref["minCOV"]) <= 1e-5 * abs(ref["minCOV"]), (t, g["minCOV"], ref["minCOV"])
    assert abs(g["mu"] - ref["mu"]) <= 1e-6 * (abs(ref["mu"]) + 10.0), (t, g["mu"], ref["mu"])
    assert abs(g["lambda_"] - ref["lambda_"]) <= 1e-4 * abs(ref["lambda_"]), (t, g["lambda_"], ref["lambda_"])
    assert abs(g["tau"] - ref["tau"]) <= 1e-4 * max(1e-12, abs(ref["tau"])), (t, g["tau"], ref["tau"])
    gh = {(i, j): E for (i, j, sc, E, p) in g["hits"]}
    rh = {(i, j): E for (i, j, sc, E, p) in ref["hits"]}
    assert set(gh) == set(rh), (t, sorted(set(gh) ^ set(rh))[:10])
    for k in rh:
        assert abs(gh[k] - rh[k]) <= 1e-4 * rh[k] + 1e-300, (t, k, gh[k], rh[k])
    sets = {}
    for cut in (10.0, 0.05):
        sets[cut] = {k for k in rh if rh[k] < cut}
        assert {k for k in gh if gh[k] < cut} == sets[cut], (t, cut)
    return len(rh), len(sets[10.0]), len(sets[0.05])


def test_rrna_scale_alignment_against_oracle(covgpu, oracle):
    s, ax, w = rrna_workload(covgpu)
    N, L = ax.shape
    ns = 20
    types = ["GTp", "MIp", "CHIp", "RAFp"]
    e = covgpu.Engine(N, L, maxslots=ns + 1, maxnull=ns)
    e.set_tree(s.parent, s.left, s.right)
    tens = e.rscape(ax, w, types, nshuffle=ns, counter=covgpu.TENSOR, thresh=THRESH)
    simt = e.rscape(ax, w, types, nshuffle=ns, counter=covgpu.SIMT, thresh=THRESH)
    e.close()
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    refs = oracle.rscape_multi(ax, w, T, types, nshuffle=ns, thresh=THRESH)
    sizes = {}
    for q, t in enumerate(types):
        sizes[t] = compare(tens[q], refs[q], t + "/tensor")
        compare(simt[q], refs[q], t + "/simt")
    print("\nrRNA scale %dx%d, pairs at E < %g, E < 10, E < 0.05: %s" % (N, L, THRESH, sizes))
    # the comparison carries weight: hundreds of pairs per statistic
    assert all(n >= 100 for n, _, _ in sizes.values()), sizes


def test_batched_nulls_against_oracle(covgpu, oracle):
    N, L, ns = 500, 400, 200
    s = covgpu.Synth(N, L, 1.5, 100, 10, 6, 14, 0.08, seed=7)
    w = covgpu.weights_pb(s.ax)
    e = covgpu.Engine(N, L, maxslots=ns + 1, maxnull=ns)
    e.set_tree(s.parent, s.left, s.right)
    g = e.rscape(s.ax, w, ["GTp"], nshuffle=ns, counter=covgpu.TENSOR, thresh=THRESH)[0]
    e.close()
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    ref = oracle.rscape(s.ax, w, T, covtype="GTp", nshuffle=ns, thresh=THRESH)
    n, n10, nsig = compare(g, ref, "GTp")
    print("\nbatched nulls %dx%d, %d nulls: pairs at E < %g, E < 10, E < 0.05: %d %d %d" % (N, L, ns, THRESH, n,
                                                                                       n10, nsig))
    assert n >= 10
