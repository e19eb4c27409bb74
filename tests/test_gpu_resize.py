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
