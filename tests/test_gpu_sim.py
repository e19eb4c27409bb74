"""The GPU P(t) simulator against the oracle and, distributionally, against
the independent host generator (needs a GB300).

Tables: every branch's P4 and P16 within 1e-12 of the oracle's
ConditionalsFromRate.  Draws: given the device's tables, the simulated
alignments are byte-identical to the oracle's (same Philox streams, same
64-bit thresholds).  Distribution: two-sample KS tests of column entropies
and of G statistics of disjoint column pairs against alignments from the
host generator on the same trees and model (independent random streams).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def setup(covgpu, N, L, seed, nbp=12):
    s = covgpu.Synth(N, L, 1.2, nbp, max(1, nbp // 6), 2, 8, 0.0, seed=seed, tree_kind=1)
    e = covgpu.Engine(N, L, maxslots=4, maxnull=3)
    e.set_tree(s.parent, s.left, s.right)
    return s, e


@pytest.mark.parametrize("N,L", [(40, 60), (150, 97), (7, 45)])
def test_tables_match_oracle(covgpu, oracle, N, L):
    s, e = setup(covgpu, N, L, 3)
    Q4, pi4, Q16, pi16 = covgpu.synth_model()
    e.simulate(s.ld, s.rd, Q4, pi4, Q16, pi16, s.ct, seed=5)
    P4, P16 = e.sim_tables()
    times = np.ravel(np.column_stack([s.ld, s.rd]))
    for b, t in enumerate(times):
        assert np.abs(P4[b] - oracle.sim_conditionals(Q4, t)).max() < 1e-12
        assert np.abs(P16[b] - oracle.sim_conditionals(Q16, t)).max() < 1e-12
    e.close()


@pytest.mark.parametrize("N,L", [(40, 60), (150, 97), (7, 45), (300, 128)])
@pytest.mark.parametrize("with_root,gaps", [(False, 0.0), (True, 0.0), (False, 0.15)])
def test_alignments_identical(covgpu, oracle, N, L, with_root, gaps):
    s, e = setup(covgpu, N, L, 11)
    Q4, pi4, Q16, pi16 = covgpu.synth_model()
    root = (np.random.default_rng(2).integers(0, 4, L)).astype(np.uint8) if with_root else None
    e.simulate(s.ld, s.rd, Q4, pi4, Q16, pi16, s.ct, root=root, gap_rate=gaps, gap_mean=3.0, seed=9, rep0=4,
               first_slot=1, nrep=3)
    P4, P16 = e.sim_tables()
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    for r in range(3):
        got = e.get_alignment(1 + r)
        ref = oracle.simulate(T, L, s.ct, P4, P16, pi4, pi16, root, gaps, 3.0, 9, 4 + r)
        assert np.array_equal(got, ref), (r, np.argwhere(got != ref)[:5])
    e.close()


def test_bad_arguments(covgpu):
    s, e = setup(covgpu, 20, 40, 1)
    Q4, pi4, Q16, pi16 = covgpu.synth_model()
    ct = s.ct.copy()
    ct[0] = 5            # partner that does not point back
    with pytest.raises(RuntimeError):
        e.simulate(s.ld, s.rd, Q4, pi4, Q16, pi16, ct)
    with pytest.raises(RuntimeError):
        e.simulate(s.ld, s.rd, Q4, pi4 * 2, Q16, pi16, s.ct)
    with pytest.raises(RuntimeError):
        e.simulate(-np.ones_like(s.ld), s.rd, Q4, pi4, Q16, pi16, s.ct)
    e.close()


def entropies(ax, cols):
    H = []
    for c in cols:
        f = np.bincount(ax[:, c], minlength=4)[:4].astype(float)
        f = f[f > 0] / f.sum()
        H.append(-(f * np.log(f)).sum())
    return H


def gstats(ax, pairs):
    G = []
    for i, j in pairs:
        C = np.zeros((4, 4))
        np.add.at(C, (ax[:, i], ax[:, j]), 1.0)
        n = C.sum()
        E = np.outer(C.sum(1), C.sum(0)) / n
        m = C > 0
        G.append(2.0 * (C[m] * np.log(C[m] / E[m])).sum())
    return G


def test_distribution_matches_host_generator(covgpu):
    stats = pytest.importorskip("scipy.stats")
    N, L = 120, 200
    Hg, Hh, Gg, Gh, Pg, Ph = [], [], [], [], [], []
    Q4, pi4, Q16, pi16 = covgpu.synth_model()
    for seed in range(12):
        s = covgpu.Synth(N, L, 1.2, 30, 5, 3, 9, 0.0, seed=100 + seed, tree_kind=1)
        e = covgpu.Engine(N, L, maxslots=2, maxnull=1)
        e.set_tree(s.parent, s.left, s.right)
        e.simulate(s.ld, s.rd, Q4, pi4, Q16, pi16, s.ct, seed=7, rep0=seed)
        g = e.get_alignment(0)
        e.close()
        unp = [c for c in range(L) if s.ct[c] < 0]
        Hg += entropies(g, unp)
        Hh += entropies(s.ax, unp)
        pairs = list(zip(unp[0::2], unp[1::2]))
        Gg += gstats(g, pairs)
        Gh += gstats(s.ax, pairs)
        bp = [(c, s.ct[c]) for c in range(L) if s.ct[c] > c]
        Pg += gstats(g, bp)
        Ph += gstats(s.ax, bp)
    for a, b, what in [(Hg, Hh, "column entropy"), (Gg, Gh, "G of unpaired pairs"), (Pg, Ph, "G of base pairs")]:
        p = stats.ks_2samp(a, b).pvalue
        assert p > 1e-3, (what, p, np.mean(a), np.mean(b))


@pytest.mark.parametrize("N,L", [(40, 60), (1200, 150), (7, 45)])
def test_device_weights_and_gapfilter(covgpu, oracle, N, L):
    s = covgpu.Synth(N, L, 1.0, 6, 1, 2, 6, 0.3, seed=4, tree_kind=1)
    ax = s.ax.copy()
    ax[0, :3] = [5, 15, 16]     # degenerate, N and '*' codes
    ax[1, 3] = 17               # '~' is skipped by the gap filter
    e = covgpu.Engine(N, L)
    e.set_alignment(0, ax)
    w = e.weights_pb(0, set=True)
    assert np.allclose(w, oracle.weights_pb(ax), rtol=1e-12, atol=0)
    if N <= 1200:
        g = e.weights_gsc(0, set=False)
        assert np.allclose(g, oracle.weights_gsc(ax), rtol=1e-10, atol=1e-13)
    for wgt in (None, w):
        for thr in (0.5, 0.75, 0.95):
            assert np.array_equal(e.gapfilter(0, wgt, thr), oracle.gapfilter(ax, wgt, thr) == 1)
    e.close()


@pytest.mark.parametrize("N,L,dup", [(300, 80, 0), (257, 33, 40), (999, 120, 200), (2, 10, 0), (4800, 20, 0)])
def test_gsc_single_launch_upgma(covgpu, oracle, N, L, dup):
    """GSC weights from the one-launch UPGMA (cached row minima) against the
    oracle, with duplicated sequences (exact distance ties, tie-breaking by
    pair order) and at the largest size that still takes this kernel."""
    s = covgpu.Synth(N, L, 0.8, 2, 1, 1, 2, 0.1, seed=N + dup, tree_kind=1)
    ax = s.ax.copy()
    rng = np.random.default_rng(N)
    for k in range(dup):               # copies of earlier rows
        i, j = rng.integers(0, N, size=2)
        ax[j] = ax[i]
    e = covgpu.Engine(N, L)
    e.set_alignment(0, ax)
    g = e.weights_gsc(0, set=False)
    e.close()
    if N <= 1200:
        assert np.allclose(g, oracle.weights_gsc(ax), rtol=1e-10, atol=1e-13)
    assert np.all(np.isfinite(g)) and abs(g.sum() - N) < 1e-6 * N
