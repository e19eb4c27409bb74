"""Helix aggregation (src/aggregate.c, src/structure.c ct_split_rmlist):
the helix split on the host against structures worked through by hand from
the reference's rules, and the aggregated p-values on the device against
scipy's chi-square distribution."""
import numpy as np
import pytest


def ct_of(db):
    """0-based partner table of a dot-bracket string ('(' ')' and '[' ']')."""
    ct = [-1] * len(db)
    st = {"(": [], "[": []}
    for j, c in enumerate(db):
        if c in "([":
            st[c].append(j)
        elif c in ")]":
            i = st["(" if c == ")" else "["].pop()
            ct[i], ct[j] = j, i
    return np.array(ct, dtype=np.int32)


@pytest.mark.parametrize("db,expect", [
    ("((((....))))", [4]),
    # one unpaired residue on each side of the inner stem: 2 <= helix_unpaired
    ("(((.((....)).)))", [5]),
    # four unpaired residues around the inner stem: a new helix
    ("((..((....))..))", [2, 2]),
    # two hairpins, then a multiloop closing stem (two faces)
    ("((((..))((..))))", [2, 2, 2]),
    ("..((...))..((...)).", [2, 2]),
    ("........", []),
])
def test_helix_split(covgpu, db, expect):
    H = covgpu.helices(ct_of(db), 2)
    assert [len(h) for h in H] == expect
    for h in H:
        assert [i for i, _ in h] == sorted(i for i, _ in h)
    ct = ct_of(db)
    assert sorted(p for h in H for p in h) == sorted((i, int(ct[i])) for i in range(len(ct)) if ct[i] > i)


def test_helix_split_order_and_unpaired_threshold(covgpu):
    db = "((((..((....))..))))"
    assert [len(h) for h in covgpu.helices(ct_of(db), 2)] == [2, 4]
    assert [len(h) for h in covgpu.helices(ct_of(db), 4)] == [6]
    # the inner hairpin is found first
    assert covgpu.helices(ct_of(db), 2)[0] == [(6, 13), (7, 12)]


def test_helix_split_rejects_pseudoknots_and_bad_tables(covgpu):
    with pytest.raises(ValueError):
        covgpu.helices(ct_of("((..[[..))..]]"), 2)
    with pytest.raises(ValueError):
        covgpu.helices(np.array([1, 2, 0], dtype=np.int32), 2)


@pytest.mark.gpu
def test_aggregation_matches_chi_square(covgpu):
    stats = pytest.importorskip("scipy.stats")
    rng = np.random.default_rng(3)
    helices = [rng.uniform(1e-9, 1.0, size=n) ** 3 for n in (1, 2, 3, 5, 8, 13, 40)]
    helices.append(np.array([1e-30, 0.5, 0.2]))
    subs = [rng.integers(0, 30, size=len(h)).astype(float) for h in helices]
    power = [rng.uniform(0, 1, size=len(h)) for h in helices]
    e = covgpu.Engine(20, 20)
    nh = len(helices)
    for method in (covgpu.AGG_FISHER, covgpu.AGG_LANCASTER, covgpu.AGG_WFISHER, covgpu.AGG_SIDAK):
        aux = subs if method == covgpu.AGG_LANCASTER else power if method == covgpu.AGG_WFISHER else None
        pagg, Eagg = e.aggregate(method, helices, aux)
        for h, p in enumerate(helices):
            n = len(p)
            if n == 1:
                ref = p[0]
            elif method == covgpu.AGG_FISHER:
                ref = stats.chi2.sf(np.sum(-2 * np.log(p)), 2 * n)
            elif method == covgpu.AGG_SIDAK:
                ref = 1 - np.exp(n * np.log(1 - p.min()))
            else:
                if method == covgpu.AGG_LANCASTER:
                    w = 1 + subs[h]
                else:
                    w = 0.01 + power[h]
                    w = w * (2 * n / w.sum())
                ref = stats.chi2.sf(np.sum(stats.chi2.isf(p, w)), w.sum())
            assert pagg[h] == pytest.approx(ref, rel=1e-7, abs=1e-300), (method, h, pagg[h], ref)
        assert np.allclose(Eagg, nh * pagg)
    with pytest.raises(RuntimeError):
        e.aggregate(covgpu.AGG_LANCASTER, helices, None)
    with pytest.raises(RuntimeError):
        e.aggregate(covgpu.AGG_FISHER, [np.array([0.5, 1.5])])
    e.close()


def test_oracle_aggregation_pinned_to_chi_square(oracle):
    """The oracle's restatement of agg_FISHER / agg_LANCASTER / agg_WFISHER /
    agg_SIDAK and of the two weight rules (src/aggregate.c:146-322, 375-488)
    against scipy's chi-square distribution and the rules written out."""
    stats = pytest.importorskip("scipy.stats")
    rng = np.random.default_rng(5)
    for n in (1, 2, 3, 7, 20):
        p = rng.uniform(1e-6, 1.0, size=n)
        subs = rng.integers(0, 40, size=n).astype(float)
        power = rng.uniform(0, 1, size=n)
        wl = oracle.agg_weights(oracle.AGG_LANCASTER, subs)
        assert np.array_equal(wl, 1.0 + subs)
        ww = oracle.agg_weights(oracle.AGG_WFISHER, power)
        assert np.allclose(ww, (0.01 + power) * 2 * n / np.sum(0.01 + power), rtol=1e-15)
        assert ww.sum() == pytest.approx(2 * n, rel=1e-14)
        if n == 1:
            for m in range(4):
                assert oracle.agg_pvalue(m, p, subs if m == 1 else power) == p[0]
            continue
        assert oracle.agg_pvalue(oracle.AGG_FISHER, p) == pytest.approx(
            stats.chi2.sf(np.sum(-2 * np.log(p)), 2 * n), rel=1e-12)
        for m, w, aux in ((oracle.AGG_LANCASTER, wl, subs), (oracle.AGG_WFISHER, ww, power)):
            ref = stats.chi2.sf(np.sum(stats.chi2.ppf(1 - p, w)), w.sum())
            assert oracle.agg_pvalue(m, p, aux) == pytest.approx(ref, rel=1e-10)
        assert oracle.agg_pvalue(oracle.AGG_SIDAK, p) == pytest.approx(1 - (1 - p.min()) ** n, rel=1e-12)
    # equal weights of 2 reduce the weighted forms to Fisher's
    p = rng.uniform(1e-3, 1.0, size=6)
    assert oracle.lib().orc_agg_weighted(6, p, np.full(6, 2.0)) == pytest.approx(
        oracle.agg_pvalue(oracle.AGG_FISHER, p), rel=1e-10)


@pytest.mark.gpu
def test_aggregation_matches_oracle(covgpu, oracle):
    """covgpu_aggregate against the oracle's restatement of the reference's
    four methods and weight rules, on p-values in [1e-6, 1) where the
    reference's lower-tail inversion at 1 - p keeps its precision."""
    rng = np.random.default_rng(11)
    helices = [rng.uniform(1e-6, 1.0, size=n) for n in (1, 2, 3, 4, 6, 9, 15, 31)]
    subs = [rng.integers(0, 30, size=len(h)).astype(float) for h in helices]
    power = [rng.uniform(0, 1, size=len(h)) for h in helices]
    e = covgpu.Engine(20, 20)
    for method in (covgpu.AGG_FISHER, covgpu.AGG_LANCASTER, covgpu.AGG_WFISHER, covgpu.AGG_SIDAK):
        aux = subs if method == covgpu.AGG_LANCASTER else power if method == covgpu.AGG_WFISHER else None
        pagg, Eagg = e.aggregate(method, helices, aux)
        for h, p in enumerate(helices):
            ref = oracle.agg_pvalue(method, p, aux[h] if aux is not None else None)
            assert pagg[h] == pytest.approx(ref, rel=1e-8, abs=1e-300), (method, h, pagg[h], ref)
        assert np.allclose(Eagg, len(helices) * pagg)
    e.close()
