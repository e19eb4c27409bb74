"""Substitutions on the tree and pair power against the oracle (needs a GB300).

Tree_Substitutions counts (nsubs, ndouble, njoin) are integers on the same
Fitch reconstruction (same random tie-break stream), so they must be equal;
the power of every pair is a step-curve lookup and must be equal too.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RECON_STREAM = 0xFFFFFFFF


@pytest.mark.parametrize("N,L", [(40, 60), (150, 97), (7, 45), (300, 130)])
@pytest.mark.parametrize("includegaps", [False, True])
def test_substitutions_match_oracle(covgpu, oracle, N, L, includegaps):
    s = covgpu.Synth(N, L, 1.5, 8, 1, 2, 8, 0.15, seed=6, tree_kind=0)
    ax = s.ax.copy()
    ax[0, :4] = [5, 15, 16, 17]      # ambiguity codes take random Fitch states
    e = covgpu.Engine(N, L, maxslots=2, maxnull=1)
    e.set_alignment(0, ax)
    e.set_tree(s.parent, s.left, s.right)
    ns, nd, nj = e.substitutions(0, seed=77, includegaps=includegaps)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    rns, rnd, rnj = oracle.substitutions(ax, T, 77, RECON_STREAM, includegaps)
    assert np.array_equal(ns, rns)
    assert np.array_equal(nd, rnd)
    assert np.array_equal(nj, rnj)
    e.close()


def test_power_matches_oracle(covgpu, oracle):
    N, L = 120, 80
    s = covgpu.Synth(N, L, 1.5, 10, 2, 2, 6, 0.1, seed=8, tree_kind=1)
    e = covgpu.Engine(N, L, maxslots=1, maxnull=0)
    e.set_alignment(0, s.ax)
    e.set_tree(s.parent, s.left, s.right)
    ns, nd, nj = e.substitutions(0, seed=3)
    rng = np.random.default_rng(1)
    curves = []
    for top in (2.0 * ns.max() + 2, nj.max() + 2, nd.max() + 2):
        subs = np.sort(rng.uniform(0, top, 25))
        prob = np.sort(rng.uniform(0, 1, 25))
        curves.append((subs, prob))
    p1, pj, pd = e.power(*curves)
    iu = np.triu_indices(L, 1)
    n1 = (ns[:, None] + ns[None, :])[iu]
    ref1 = [oracle.power_step(x, *curves[0]) for x in n1]
    refj = [oracle.power_step(x, *curves[1]) for x in nj[iu]]
    refd = [oracle.power_step(x, *curves[2]) for x in nd[iu]]
    assert np.array_equal(p1, ref1) and np.array_equal(pj, refj) and np.array_equal(pd, refd)
    # curves not given: 0 for single, -1 for join and double
    q1, qj, qd = e.power(single=curves[0])
    assert np.array_equal(q1, ref1) and np.all(qj == -1.0) and np.all(qd == -1.0)
    e.close()


def classes_of(pp, L):
    """power_SPAIR_AddMI (src/power.c:201-218) on pair probabilities pp[L][L][16]."""
    iu = np.triu_indices(L, 1)
    p = pp[iu]
    w = ((p[:, 3] + p[:, 12]) + p[:, 6]) + p[:, 9]
    g = p[:, 11] + p[:, 14]
    return w, g, (1.0 - w) - g


@pytest.mark.parametrize("N,L", [(60, 70), (400, 130)])
def test_pair_classes_match_host_pp_and_oracle(covgpu, oracle, N, L):
    """The device pair classes equal those computed from the host pair
    probabilities the drop-in fills (same FP64 operations), and those of the
    oracle's pair probabilities within 2e-9 (the counts are of 33-bit
    quantised weights)."""
    s = covgpu.Synth(N, L, 1.5, L // 6, 2, 5, 12, 0.1, seed=N + L)
    w = covgpu.weights_pb(s.ax) * np.random.default_rng(3).uniform(0.7, 1.3, N)
    e = covgpu.Engine(N, L)
    e.set_weights(w)
    e.set_alignment(0, s.ax)
    for counter in (covgpu.SIMT, covgpu.TENSOR):
        e.score(["GT"], counter=counter)
        got = e.pair_classes(0)
        pp = e.get_probs(0, w)[0]
        for g, h in zip(got, classes_of(pp, L)):
            assert np.array_equal(g, h)
        ref = classes_of(oracle.probs(s.ax, w)[0], L)
        for g, h in zip(got, ref):
            assert np.max(np.abs(g - h)) <= 2e-9
    e.close()
