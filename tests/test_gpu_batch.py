"""The E-valued path over a batch of ragged families (covgpu_rscape_families:
every device pass one grouped launch over all families, the passes from the
nulls to the corrected scores a CUDA graph) against covgpu_rscape run family
by family, and against the FP64 oracle's restatement of null_rscape +
cov_CreateHitList (src/R-scape.c:1614-1724, src/covariation.c:778-1006).
Needs a GB300.

Families differ in N (20 .. 1,200: GSC and position-based weights under
R-scape's rule, src/R-scape.c:1545-1562), L (45 .. 260: 20 or 200 nulls under
R-scape's null count rule, src/R-scape.c:2449-2456) and tree.  A batch family
gets the same nulls (same seed), counts, statistics and histograms as the
single-family call; the tail fit runs the same search on one block instead
of a grid, so lambda and tau agree to the search's convergence (1e-6), not
to the bit.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (N, L, seed): GSC (N <= 1000) and position-based (N > 1000) weights; L < 50
# takes 200 nulls
SIZES = [(20, 120, 11), (45, 260, 12), (130, 60, 13), (300, 45, 14), (64, 200, 15), (700, 90, 16),
         (1200, 70, 17), (33, 150, 18), (250, 33 + 64, 19)]


def family(covgpu, N, L, seed, tree_len=1.8, frac=0.25):
    nbp = max(1, int(round(frac * L / 2)))
    nhelix = max(1, -(-nbp // 8))
    hmin = min(4, nbp // nhelix)
    return covgpu.Synth(N, L, tree_len, nbp, nhelix, hmin, 12, 0.08, 3.0, seed=seed)


def single(covgpu, s, types, wgt=None, **kw):
    N, L = s.ax.shape
    ns = 300 if L < 40 else (200 if L < 50 or N * L < 1000 else 20)
    e = covgpu.Engine(N, L, maxslots=ns + 1, maxnull=ns)
    e.set_tree(s.parent, s.left, s.right)
    e.set_alignment(0, s.ax)
    if wgt is None:
        if N <= 1000:
            e.weights_gsc(0, set=True)
        else:
            e.weights_pb(0, set=True)
    else:
        e.set_weights(wgt)
    r = e.rscape(None, None, types, hitcap=1 << 12, **kw)
    single.launches += e.last_timing()[1]
    e.close()
    return r


single.launches = 0


def same(g, r, tag):
    assert g["status"] == r["status"], tag
    assert g["nshuffle"] == r["nshuffle"], tag
    if r["status"]:
        return
    for k in ("w", "minCOV", "maxCOV", "null_minCOV", "null_maxCOV", "h_phi", "mu"):
        assert abs(g[k] - r[k]) <= 1e-12 * max(1.0, abs(r[k])), (tag, k, g[k], r[k])
    for k in ("h_nb", "h_imin", "h_imax", "h_cmin", "h_n", "h_Nc", "h_No", "Nt"):
        assert g[k] == r[k], (tag, k, g[k], r[k])
    for k in ("lambda_", "tau"):
        assert abs(g[k] - r[k]) <= 1e-6 * abs(r[k]), (tag, k, g[k], r[k])
    gh = {(i, j): E for (i, j, sc, E, p) in g["hits"]}
    rh = {(i, j): E for (i, j, sc, E, p) in r["hits"]}
    # a pair whose E-value sits within the fits' agreement of the threshold
    # may fall on either side of it
    edge = {k for k in set(gh) ^ set(rh) if abs((gh.get(k) or rh.get(k)) - 10.0) <= 1e-4 * 10.0}
    assert set(gh) ^ set(rh) <= edge, (tag, sorted(set(gh) ^ set(rh))[:10])
    for k in set(gh) & set(rh):
        assert abs(gh[k] - rh[k]) <= 1e-4 * rh[k] + 1e-300, (tag, k, gh[k], rh[k])


def test_batch_matches_single_family_calls(covgpu):
    fams = [family(covgpu, N, L, seed) for N, L, seed in SIZES]
    types = ["GTp", "MIp", "CHIp"]
    b = covgpu.Batch()
    got = b.rscape([dict(ax=s.ax, parent=s.parent, left=s.left, right=s.right) for s in fams], types,
                   counter=covgpu.TENSOR, thresh=10.0)
    ms_dev, ms_rest, ms_host, nl, nch = b.timing()
    npairs = 0
    single.launches = 0
    for k, s in enumerate(fams):
        ref = single(covgpu, s, types, counter=covgpu.TENSOR, thresh=10.0)
        for q, t in enumerate(types):
            same(got[k][q], ref[q], (k, t))
            npairs += len(ref[q]["hits"])
    # the comparison carries weight: pairs with E < 10 in most families
    assert npairs >= 50, npairs
    # one grouped launch per pass: far fewer than the families' own launches
    assert nl < single.launches / 2, (nl, single.launches)
    b.close()


def test_batch_simt_raf_rafs_and_given_weights(covgpu):
    fams = [family(covgpu, N, L, seed) for N, L, seed in SIZES[:5]]
    rng = np.random.default_rng(5)
    wts = [covgpu.weights_pb(s.ax) * rng.uniform(0.7, 1.3, s.ax.shape[0]) for s in fams]
    types = ["CHIp", "RAFp", "RAFSp", "GT"]
    b = covgpu.Batch()
    got = b.rscape([dict(ax=s.ax, parent=s.parent, left=s.left, right=s.right, wgt=w) for s, w in zip(fams, wts)],
                   types, counter=covgpu.SIMT, thresh=10.0)
    for k, s in enumerate(fams):
        ref = single(covgpu, s, types, wgt=wts[k], counter=covgpu.SIMT, thresh=10.0)
        for q, t in enumerate(types):
            same(got[k][q], ref[q], (k, t))
    b.close()


def test_batch_chunks_and_graph_replay_give_the_same_results(covgpu):
    fams = [family(covgpu, N, L, seed) for N, L, seed in SIZES]
    fl = [dict(ax=s.ax, parent=s.parent, left=s.left, right=s.right) for s in fams]
    b1 = covgpu.Batch()
    one = b1.rscape(fl, ["GTp"], counter=covgpu.TENSOR, thresh=10.0)
    assert b1.timing()[4] == 1
    again = b1.rscape(fl, ["GTp"], counter=covgpu.TENSOR, thresh=10.0)   # the captured graph, replayed
    b1.close()
    b2 = covgpu.Batch(mem_gb=0.02)    # a budget that forces several chunks
    many = b2.rscape(fl, ["GTp"], counter=covgpu.TENSOR, thresh=10.0)
    assert b2.timing()[4] > 1, b2.timing()
    b2.close()
    for k in range(len(fams)):
        for other in (again, many):
            a, c = one[k][0], other[k][0]
            for key in a:
                assert a[key] == c[key], (k, key, a[key], c[key])


def test_batch_against_oracle(covgpu, oracle):
    fams = [family(covgpu, N, L, seed) for N, L, seed in [(100, 120, 21), (260, 80, 22), (60, 140, 23)]]
    ws = [covgpu.weights_pb(s.ax) for s in fams]
    b = covgpu.Batch()
    got = b.rscape([dict(ax=s.ax, parent=s.parent, left=s.left, right=s.right, wgt=w) for s, w in zip(fams, ws)],
                   ["GTp"], counter=covgpu.TENSOR, thresh=10.0)
    b.close()
    nhit = 0
    for k, s in enumerate(fams):
        T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
        ref = oracle.rscape(s.ax, ws[k], T, covtype="GTp", nshuffle=20, thresh=10.0)
        g = got[k][0]
        assert abs(g["w"] - ref["w"]) <= 1e-7 * abs(ref["w"])
        for key in ("h_nb", "h_imin", "h_imax", "h_cmin", "h_n", "h_Nc", "h_No"):
            assert g[key] == ref[key], (k, key)
        assert abs(g["lambda_"] - ref["lambda_"]) <= 1e-4 * abs(ref["lambda_"])
        gh = {(i, j): E for (i, j, sc, E, p) in g["hits"]}
        rh = {(i, j): E for (i, j, sc, E, p) in ref["hits"]}
        assert set(gh) == set(rh), (k, sorted(set(gh) ^ set(rh))[:10])
        for key in rh:
            assert abs(gh[key] - rh[key]) <= 1e-4 * rh[key] + 1e-300
        nhit += len(rh)
    assert nhit >= 10, nhit


def test_batch_reports_the_bad_family(covgpu):
    fams = [family(covgpu, N, L, seed) for N, L, seed in SIZES[:3]]
    fl = [dict(ax=s.ax, parent=s.parent, left=s.left, right=s.right) for s in fams]
    bad = dict(fl[1])
    bad["left"] = np.array(fams[1].left, dtype=np.int32).copy()
    bad["left"][0] = bad["left"][1]     # a node listed twice
    b = covgpu.Batch()
    with pytest.raises(RuntimeError, match="family 1"):
        b.rscape([fl[0], bad, fl[2]], ["GTp"])
    ax = fams[2].ax.copy()
    ax[0, 0] = 99
    with pytest.raises(RuntimeError, match="family 2"):
        b.rscape([fl[0], fl[1], dict(fl[2], ax=ax)], ["GTp"])
    # the batch still works afterwards
    r = b.rscape(fl, ["GTp"], counter=covgpu.TENSOR)
    assert len(r) == 3
    b.close()


def test_batch_schedules_give_the_same_results(covgpu):
    """The count schedule (which families the SIMT kernel counts, the tensor
    count's raster order) changes no result: the two counters give the same
    counts.  The autotuner returns one of its candidates."""
    fams = [family(covgpu, N, L, seed) for N, L, seed in SIZES]
    fl = [dict(ax=s.ax, parent=s.parent, left=s.left, right=s.right) for s in fams]
    b = covgpu.Batch()
    ref = b.rscape(fl, ["GTp", "CHIp"], counter=covgpu.TENSOR, thresh=10.0)
    # all tensor, all SIMT, mixed; square and band rasters
    for thr, sb in ((0, 4), (1 << 20, 10), (300, 16), (0, 32004), (300, 6003)):
        b.set_schedule(thr, sb)
        got = b.rscape(fl, ["GTp", "CHIp"], counter=covgpu.TENSOR, thresh=10.0)
        for k in range(len(fams)):
            for q in range(2):
                for key in ref[k][q]:
                    assert got[k][q][key] == ref[k][q][key], (thr, sb, k, q, key)
    bt, bs, times = b.autotune(fl[:5], ["GTp"], thr=(0, 200), sb=(6, 10), counter=covgpu.TENSOR)
    assert len(times) == 4 and (bt, bs) in times
    assert times[(bt, bs)] == min(times.values())
    b.close()


def test_batch_edge_families_and_raf_only(covgpu):
    """Families of one, two and three sequences in a batch with ordinary
    ones, against per-family calls; and a batch asked for RAF alone (no
    weighted counts at all)."""
    rng = np.random.default_rng(3)
    fams = [family(covgpu, 40, 90, 31), family(covgpu, 3, 60, 32), family(covgpu, 2, 55, 33),
            family(covgpu, 150, 70, 34)]
    one = rng.integers(0, 4, size=(1, 80)).astype(np.uint8)
    fl = [dict(ax=s.ax, parent=s.parent, left=s.left, right=s.right) for s in fams]
    fl.insert(1, dict(ax=one))
    b = covgpu.Batch()
    got = b.rscape(fl, ["GTp"], counter=covgpu.TENSOR, thresh=10.0)
    assert got[1][0]["status"] == 2 and got[1][0]["nshuffle"] == 0
    for k, s in ((0, fams[0]), (2, fams[1]), (3, fams[2]), (4, fams[3])):
        N, L = s.ax.shape
        ns = 300 if (N < 4 or L < 40) else (200 if (L < 50 or N * L < 1000) else 20)
        e = covgpu.Engine(N, L, maxslots=ns + 1, maxnull=ns)
        e.set_tree(s.parent, s.left, s.right)
        e.set_alignment(0, s.ax)
        e.weights_gsc(0, set=True)
        ref = e.rscape(None, None, ["GTp"], hitcap=1 << 12, counter=covgpu.TENSOR, thresh=10.0)[0]
        e.close()
        same(got[k][0], ref, (k, N, L))
    raf = b.rscape(fl, ["RAFp", "RAF"], counter=covgpu.TENSOR, thresh=10.0)
    both = b.rscape(fl, ["RAFp", "GTp"], counter=covgpu.TENSOR, thresh=10.0)
    for k in (0, 2, 3, 4):
        for key in raf[k][0]:
            assert raf[k][0][key] == both[k][0][key], (k, key)
    b.close()
