"""A context resized between families gives what a context made for each
family's exact size gives (scores, null fit, E-values), on both counting
paths and for every order of sizes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FAMILIES = [(300, 150, 11), (90, 61, 12), (420, 197, 13), (40, 33, 14), (300, 150, 11)]


def run(e, covgpu, N, L, seed, counter):
    nbp = max(2, L // 10)
    s = covgpu.Synth(N, L, 1.4, nbp, 1 if nbp < 4 else 2, 2, 12, 0.08, seed=seed)
    e.set_tree(s.parent, s.left, s.right)
    w = covgpu.weights_pb(s.ax)
    r = e.rscape(s.ax, w, ["GTp", "RAFp"], nshuffle=6, counter=counter, thresh=10.0)
    cov = np.zeros(L * L)
    covgpu.lib().covgpu_get_cov(e.h, 0, 0, cov)
    return r, cov


@pytest.mark.parametrize("counter", ["tensor", "simt"])
def test_resize_matches_fresh_contexts(covgpu, counter):
    c = covgpu.TENSOR if counter == "tensor" else covgpu.SIMT
    big = covgpu.Engine(420, 197, maxslots=7, maxnull=6)
    for (N, L, seed) in FAMILIES:
        big.resize(N, L)
        r1, cov1 = run(big, covgpu, N, L, seed, c)
        fresh = covgpu.Engine(N, L, maxslots=7, maxnull=6)
        r2, cov2 = run(fresh, covgpu, N, L, seed, c)
        fresh.close()
        assert np.array_equal(cov1, cov2), (N, L)
        for a, b in zip(r1, r2):
            for k in ("w", "mu", "lambda_", "tau", "maxCOV", "minCOV", "nhit", "h_nb", "h_cmin"):
                assert a[k] == b[k], (N, L, k, a[k], b[k])
            assert a["hits"] == b["hits"]
    big.close()


def test_resize_rejects_larger_sizes(covgpu):
    e = covgpu.Engine(100, 80)
    with pytest.raises(RuntimeError):
        e.resize(101, 80)
    with pytest.raises(RuntimeError):
        e.resize(100, 81)
    e.close()


def test_autotuned_schedule_gives_identical_scores(covgpu):
    """The autotuner only reorders the count kernel's tiles: every score is
    bit-identical whatever raster it picks."""
    N, L = 500, 700
    s = covgpu.Synth(N, L, 1.4, 60, 6, 6, 12, 0.08, seed=5)
    e = covgpu.Engine(N, L, maxslots=3, maxnull=2)
    e.set_tree(s.parent, s.left, s.right)
    e.set_weights(covgpu.weights_pb(s.ax))
    e.set_alignment(0, s.ax)
    e.make_nulls(42, 0, 2, 1)
    types = ["GTp", "MIp", "RAFp"]   # RAF: the unit-weight kernel's column-pair order
    e.score(types, nslots=3, counter=covgpu.TENSOR)
    before = [e.get_cov(k, q) for k in range(3) for q in range(3)]
    best, ms = e.autotune(3, candidates=(2, 5, 10, 23, 32004, 6003))
    assert best in (2, 5, 10, 23, 32004, 6003) and all(v > 0 for v in ms.values())
    # the autotuner's choice, then every square and band schedule forced alone
    for cand in (None, 2, 23, 32004, 6003, 96002, 1001):
        if cand is not None:
            assert e.autotune(3, candidates=(cand,))[0] == cand
        e.score(types, nslots=3, counter=covgpu.TENSOR)
        after = [e.get_cov(k, q) for k in range(3) for q in range(3)]
        for a, b in zip(before, after):
            assert np.array_equal(a, b), cand
    e.close()
