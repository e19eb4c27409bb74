"""The reference-named entry points (rscape_cov.h) driven the way R-scape's
null_rscape / rscape_for_msa drive them (src/R-scape.c:1614-1724, 2502),
checked against the CPU oracle (needs a GB300)."""
import ctypes as C

import numpy as np
import pytest

from parity_tol import stat_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def abi(covgpu):
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location("rscape_abi", os.path.join(os.path.dirname(covgpu.LIBPATH),
                                                                               "rscape_abi.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize("device_resident", [0, 1])
@pytest.mark.parametrize("covtype", ["GTp", "MIp", "RAFp"])
def test_dropin_rscape_flow(covgpu, oracle, abi, covtype, device_resident):
    """The flow in the reference's host-array mode, and in device-resident mode
    (pp and the score matrix stay on the device; corr_SyncHost brings COV
    back): the same hits, E-values and scores as the oracle in both."""
    lib = abi.setup_lib(covgpu.LIBPATH)
    N, L, ns = 160, 90, 6
    s = covgpu.Synth(N, L, 1.5, 18, 2, 9, 9, 0.08, seed=21, tree_kind=1)
    w = covgpu.weights_pb(s.ax)
    code = covgpu.covtype_code(covtype)
    abc = abi.Alphabet(1, 4, 18)
    mi = lib.corr_Create(L, N, 0, 8, 50, C.byref(abc), 3)
    mi.contents.device_resident = device_resident
    errbuf = C.create_string_buffer(256)
    th = abi.Thresh(0, 0.05, 0.0, 0.0)
    rnd = abi.Rand(42)
    data = abi.Data(C.pointer(rnd), 3, None, None, mi, C.pointer(th), 1, 0, abi.RANSS, code, N, -1.0, -10.0, 0.05,
                    1.0, 0.0005, 0, 0.0, 0.0, 0.0, None, 1e-6, 0, C.cast(errbuf, C.c_char_p))
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    nulls = [abi.MsaHolder(oracle.null_msa(s.ax, T, 42, k), w, abc) for k in range(ns)]
    real = abi.MsaHolder(s.ax, w, abc)
    rl, hl, cum = abi.rscape_flow(lib, mi, nulls, real, data, code)
    got = sorted((hl.contents.hit[k].i, hl.contents.hit[k].j) for k in range(hl.contents.nhit))
    ref = oracle.rscape(s.ax, w, T, covtype=covtype, nshuffle=ns, want_matrices=True)
    exp = sorted((i, j) for (i, j, sc, E, p) in ref["hits"])
    assert got == exp
    assert abs(data.w - ref["w"]) <= 1e-6 * ref["w"]
    ev = {(hl.contents.hit[k].i, hl.contents.hit[k].j): hl.contents.hit[k].Eval for k in range(hl.contents.nhit)}
    for (i, j, sc, E, p) in ref["hits"]:
        assert abs(ev[(i, j)] - E) <= 1e-5 * E
    assert abs(mi.contents.maxCOV - ref["maxCOV"]) <= 1e-5 * abs(ref["maxCOV"])
    if device_resident:
        assert lib.corr_SyncHost(mi, errbuf) == 0, errbuf.value
    else:
        # mi->Eval holds every pair's E-value
        Ev = np.ctypeslib.as_array(mi.contents.Eval.contents.mx[0], shape=(L * L,)).reshape(L, L)
        assert np.all(Ev[np.triu_indices(L, 1)] > 0)
        if covtype != "RAFp":
            # pp and nseff on the host are the given alignment's (the nulls',
            # shuffled, stayed on the device)
            opp, one, ong, opm, ops = oracle.probs(s.ax, w)
            iu = np.triu_indices(L, 1)
            ne = np.ctypeslib.as_array(mi.contents.nseff[0], shape=(L * L,)).reshape(L, L)
            ppp = C.cast(mi.contents.pp, C.POINTER(C.POINTER(C.POINTER(C.c_double))))
            pp = np.ctypeslib.as_array(ppp[0][0], shape=(L * L * 16,)).reshape(L, L, 16)
            assert np.allclose(ne[iu], one[iu], rtol=1e-9)
            assert np.allclose(pp[iu], opp[iu], rtol=1e-6, atol=1e-15)
    # mi->COV: the corrected scores
    cov = np.ctypeslib.as_array(mi.contents.COV.contents.mx[0], shape=(L * L,)).reshape(L, L)
    iu = np.triu_indices(L, 1)
    ok, rel, small = stat_close(cov[iu], ref["COV"][iu])
    assert ok, (rel, small)
    lib.cov_FreeHitList(hl)
    lib.cov_FreeRankList(rl)
    lib.cov_FreeRankList(cum)
    lib.corr_Destroy(mi)


@pytest.mark.parametrize("device_resident", [0, 1])
def test_dropin_probs_and_statistic(covgpu, oracle, abi, device_resident):
    """corr_Probs, corr_CalculateGT and corr_CalculateCOVCorrected one by one;
    in device-resident mode corr_ValidateProbs runs on the device and
    corr_SyncHost brings the corrected scores back."""
    lib = abi.setup_lib(covgpu.LIBPATH)
    N, L = 70, 55
    s = covgpu.Synth(N, L, 1.5, 9, 1, 9, 9, 0.08, seed=4, tree_kind=1)
    w = covgpu.weights_pb(s.ax)
    abc = abi.Alphabet(1, 4, 18)
    mi = lib.corr_Create(L, N, 0, 8, 50, C.byref(abc), 3)
    mi.contents.device_resident = device_resident
    errbuf = C.create_string_buffer(256)
    m = abi.MsaHolder(s.ax, w, abc)
    assert lib.corr_Probs(None, C.byref(m.msa), None, None, mi, 0, 1e-6, 0, errbuf) == 0, errbuf.value
    opp, one, ong, opm, ops = oracle.probs(s.ax, w)
    pm = np.ctypeslib.as_array(mi.contents.pm[0], shape=(L * 4,)).reshape(L, 4)
    ne = np.ctypeslib.as_array(mi.contents.nseff[0], shape=(L * L,)).reshape(L, L)
    iu = np.triu_indices(L, 1)
    assert np.allclose(pm, opm, rtol=1e-9)
    if device_resident:
        assert np.all(ne == 0.0)          # nseff stays on the device
    else:
        assert np.allclose(ne[iu], one[iu], rtol=1e-9)
    th = abi.Thresh(0, 0.05, 0.0, 0.0)
    data = abi.Data(None, 3, None, None, mi, C.pointer(th), 1, 0, abi.GIVSS, 4, N, -1.0, -10.0, 0.05, 1.0, 0.0005, 0,
                    0.0, 0.0, 0.0, None, 1e-6, 0, C.cast(errbuf, C.c_char_p))
    assert lib.corr_CalculateGT(3, C.byref(data)) == 0
    assert lib.corr_CalculateCOVCorrected(0, C.byref(data), 0) == 0
    if device_resident:
        assert lib.corr_SyncHost(mi, errbuf) == 0, errbuf.value
    cov = np.ctypeslib.as_array(mi.contents.COV.contents.mx[0], shape=(L * L,)).reshape(L, L)
    ref, (rmin, rmax) = oracle.cov_calculate("GTp", s.ax, w)
    ok, rel, small = stat_close(cov[iu], ref[iu])
    assert ok, (rel, small)
    assert mi.contents.type == 4
    assert abs(mi.contents.maxCOV - rmax) <= 1e-5 * abs(rmax)
    lib.corr_Destroy(mi)


@pytest.mark.parametrize("device_resident", [0, 1])
@pytest.mark.parametrize("variant", ["two_set", "structured", "two_set_structured", "pdb_two_set", "wc_two_set"])
def test_dropin_two_set_and_structured(covgpu, oracle, abi, variant, device_resident):
    """R-scape -s (the two-set test: the structure's base pairs against the
    other pairs), --structured (expBP) and a PDB map with its distance rule
    through the drop-in flow: the same hits, E-values, numbers of tests,
    thresholds and contact types as the oracle."""
    lib = abi.setup_lib(covgpu.LIBPATH)
    N, L, ns = 160, 90, 6
    s = covgpu.Synth(N, L, 1.5, 18, 2, 9, 9, 0.08, seed=21, tree_kind=1)
    w = covgpu.weights_pb(s.ax)
    code = covgpu.covtype_code("GTp")
    bps = [(i, int(s.ct[i])) for i in range(L) if s.ct[i] > i]
    # the planted pairs, one of them listed first as a non-canonical type;
    # one pair listed first as STACKED and then as WWc; a contact with i > j,
    # which the reference never matches
    contacts = [(bps[0][0] + 1, bps[0][1] + 1, 5)]
    contacts += [(i + 1, j + 1, abi.WWc) for i, j in bps]
    extra = (2, 9) if (1, 8) not in bps else (3, 11)
    contacts += [(extra[0], extra[1], abi.STACKED), (extra[0], extra[1], abi.WWc), (40, 12, abi.WWc)]
    sample = {"two_set": abi.SAMPLE_BP, "structured": abi.SAMPLE_ALL, "two_set_structured": abi.SAMPLE_BP,
              "pdb_two_set": abi.SAMPLE_CONTACTS, "wc_two_set": abi.SAMPLE_WC}[variant]
    expBP = 6.5 if "structured" in variant else -1.0
    mind = 4 if variant.startswith("pdb") else 0
    m2p = np.arange(L, dtype=np.int32) if mind else None
    abc = abi.Alphabet(1, 4, 18)
    mi = lib.corr_Create(L, N, 0, 8, 50, C.byref(abc), 3)
    mi.contents.device_resident = device_resident
    errbuf = C.create_string_buffer(256)
    th = abi.Thresh(0, 0.05, 0.0, 0.0)
    rnd = abi.Rand(42)
    cl = abi.make_clist(contacts, mind)
    data = abi.Data(C.pointer(rnd), sample, None, None, mi, C.pointer(th), 1, 0, abi.RANSS, code, N, expBP, -10.0,
                    0.05, 1.0, 0.0005, 0, 0.0, 0.0, 0.0, None, 1e-6, 0, C.cast(errbuf, C.c_char_p), C.pointer(cl),
                    m2p.ctypes.data_as(C.POINTER(C.c_int)) if m2p is not None else None)
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    nulls = [abi.MsaHolder(oracle.null_msa(s.ax, T, 42, k), w, abc) for k in range(ns)]
    real = abi.MsaHolder(s.ax, w, abc)
    rl, hl, cum = abi.rscape_flow(lib, mi, nulls, real, data, code)
    kw = dict(covtype="GTp", nshuffle=ns, want_matrices=True, samplesize=sample, contacts=contacts, expBP=expBP)
    if mind:
        kw.update(msa2pdb=m2p, mind=mind)
    ref = oracle.rscape(s.ax, w, T, **kw)
    H = hl.contents
    assert H.Nt == ref["Nt"] and H.Nb == ref["Nb"]
    if sample != abi.SAMPLE_ALL:
        assert H.Nb > 0
    got = {(H.hit[k].i, H.hit[k].j): H.hit[k] for k in range(H.nhit)}
    exp = {(i, j): E for (i, j, sc, E, p) in ref["hits"]}
    assert sorted(got) == sorted(exp)
    for k, E in exp.items():
        assert abs(got[k].Eval - E) <= 1e-5 * E
    first = {}
    for (i, j, t) in contacts:
        if 1 <= i < j <= L:
            first.setdefault((i - 1, j - 1), t)
    for k, h in got.items():
        assert h.bptype == first.get(k, abi.BPNONE)
    assert abs(th.sc_bp - ref["sc_thresh"]) <= 1e-5 * abs(ref["sc_thresh"]) + 1e-9
    assert abs(th.sc_nbp - ref["sc_nbp"]) <= 1e-5 * abs(ref["sc_nbp"]) + 1e-9
    # mi->Eval (host-array mode): every pair's E-value with its own number of tests
    if not device_resident:
        Ev = np.ctypeslib.as_array(mi.contents.Eval.contents.mx[0], shape=(L * L,)).reshape(L, L)
        iu = np.triu_indices(L, 1)
        fin = np.isfinite(ref["Eval"][iu]) & (ref["Eval"][iu] > 0)
        assert np.allclose(Ev[iu][fin], ref["Eval"][iu][fin], rtol=1e-5, atol=0)
    lib.cov_FreeHitList(hl)
    lib.cov_FreeRankList(rl)
    lib.cov_FreeRankList(cum)
    lib.corr_Destroy(mi)
