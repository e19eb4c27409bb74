"""The simulator's oracle: ratematrix_ConditionalsFromRate rules
(src/ratematrix.c:185-233), inverse-CDF thresholds and the evolution
(src/cov_simulate.c:288-324,586-798) on the CPU."""
import numpy as np
import pytest


def k80(kappa=2.0):
    Q = np.full((4, 4), 0.25)
    for a, b in [(0, 2), (2, 0), (1, 3), (3, 1)]:
        Q[a, b] = 0.25 * kappa
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(1))
    return Q / np.mean(-np.diag(Q))


def test_conditionals_match_expm(oracle):
    scipy_linalg = pytest.importorskip("scipy.linalg")
    Q = k80()
    for t in [1e-6, 0.01, 0.3, 2.0, 25.0]:
        P = oracle.sim_conditionals(Q, t)
        assert np.allclose(P, scipy_linalg.expm(t * Q), rtol=0, atol=1e-13)
        assert np.allclose(P.sum(1), 1.0, rtol=0, atol=1e-15)


def test_conditionals_time_rules(oracle):
    Q = k80()
    # time 0: the reference's 1e-4 substitution is overwritten by the cap's else branch
    assert np.array_equal(oracle.sim_conditionals(Q, 0.0), np.eye(4))
    # tiny negative times become 1e-5
    assert np.allclose(oracle.sim_conditionals(Q, -1e-7), oracle.sim_conditionals(Q, 1e-5), rtol=0, atol=0)
    with pytest.raises(RuntimeError):
        oracle.sim_conditionals(Q, -0.1)
    # times above 1e4 are capped
    assert np.array_equal(oracle.sim_conditionals(Q, 5e4), oracle.sim_conditionals(Q, 1e4))


def test_cdf_thresholds(oracle):
    P = np.array([[0.5, 0.25, 0.25, 0.0], [0.0, 0.0, 0.0, 1.0]])
    C = oracle.sim_cdf(P)
    assert C[0, 0] == np.uint64(1 << 63) and C[0, 1] == np.uint64(3 << 62)
    assert C[0, 3] == np.iinfo(np.uint64).max and C[0, 2] == np.iinfo(np.uint64).max
    assert C[1, 0] == 0 and C[1, 3] == np.iinfo(np.uint64).max


def star_tree(N, bl):
    """caterpillar tree in Easel numbering: node v has internal child v+1 and leaf -v"""
    left = np.array([-(v) for v in range(N - 1)], dtype=np.int32)
    right = np.array([v + 1 if v < N - 2 else -(N - 1) for v in range(N - 1)], dtype=np.int32)
    parent = np.array([-1] + list(range(N - 2)), dtype=np.int32)
    return parent, left, right, np.full(N - 1, bl), np.full(N - 1, bl)


def test_simulate_invariants(oracle):
    N, L = 12, 40
    parent, left, right, ld, rd = star_tree(N, 0.2)
    T = oracle.TreeArrays(parent, left, right, ld, rd)
    ct = -np.ones(L, dtype=np.int32)
    for i, j in [(0, 9), (1, 8), (20, 35)]:
        ct[i], ct[j] = j, i
    Q4 = k80()
    pi4 = np.full(4, 0.25)
    Q16 = np.kron(Q4, np.eye(4)) + np.kron(np.eye(4), Q4)   # independent sites
    pi16 = np.full(16, 1 / 16)
    P4 = np.array([oracle.sim_conditionals(Q4, t) for t in np.ravel(np.column_stack([ld, rd]))])
    P16 = np.array([oracle.sim_conditionals(Q16, t) for t in np.ravel(np.column_stack([ld, rd]))])
    a = oracle.simulate(T, L, ct, P4, P16, pi4, pi16, None, 0.0, 0.0, 7, 0)
    assert a.shape == (N, L) and a.max() <= 3
    b = oracle.simulate(T, L, ct, P4, P16, pi4, pi16, None, 0.0, 0.0, 7, 0)
    assert np.array_equal(a, b)
    c = oracle.simulate(T, L, ct, P4, P16, pi4, pi16, None, 0.0, 0.0, 7, 1)
    assert not np.array_equal(a, c)
    # zero-length branches copy the root
    Z = oracle.TreeArrays(parent, left, right, np.zeros(N - 1), np.zeros(N - 1))
    root = np.arange(L, dtype=np.uint8) % 4
    I4 = np.tile(np.eye(4), (2 * (N - 1), 1, 1))
    I16 = np.tile(np.eye(16), (2 * (N - 1), 1, 1))
    z = oracle.simulate(Z, L, ct, I4, I16, pi4, pi16, root, 0.0, 0.0, 7, 0)
    assert np.array_equal(z, np.tile(root, (N, 1)))
    # gaps: about gap_rate of the cells
    g = oracle.simulate(T, 4000, -np.ones(4000, dtype=np.int32), P4, P16, pi4, pi16, None, 0.2, 3.0, 9, 0)
    assert abs(np.mean(g == 4) - 0.2) < 0.03
