"""The reference-named entry points (rscape_cov.h) driven the way R-scape's
null_rscape / rscape_for_msa drive them (src/R-scape.c:1614-1724, 2502),
checked against the CPU oracle (needs a GB300)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class Alphabet(C.Structure):
    _fields_ = [("type", C.c_int), ("K", C.c_int), ("Kp", C.c_int)]


class Msa(C.Structure):
    _fields_ = [("ax", C.POINTER(C.POINTER(C.c_uint8))), ("wgt", C.POINTER(C.c_double)), ("nseq", C.c_int),
                ("alen", C.c_int64), ("abc", C.POINTER(Alphabet))]


class DMatrix(C.Structure):
    _fields_ = [("mx", C.POINTER(C.POINTER(C.c_double))), ("n", C.c_int), ("m", C.c_int)]


class Hist(C.Structure):
    _fields_ = [("xmin", C.c_double), ("xmax", C.c_double), ("n", C.c_uint64), ("obs", C.POINTER(C.c_uint64)),
                ("bmin", C.c_double), ("bmax", C.c_double), ("w", C.c_double), ("imin", C.c_int), ("imax", C.c_int),
                ("nb", C.c_int), ("phi", C.c_double), ("cmin", C.c_int), ("Nc", C.c_uint64), ("No", C.c_uint64)]


class Mutual(C.Structure):
    _fields_ = [("alen", C.c_int64), ("nseq", C.c_int64), ("pp", C.c_void_p), ("pm", C.POINTER(C.POINTER(C.c_double))),
                ("nseff", C.POINTER(C.POINTER(C.c_double))), ("ps", C.c_void_p), ("ngap", C.c_void_p),
                ("type", C.c_int), ("class_", C.c_int), ("COV", C.POINTER(DMatrix)), ("Eval", C.POINTER(DMatrix)),
                ("besthreshCOV", C.c_double), ("minCOV", C.c_double), ("maxCOV", C.c_double), ("ishuffled", C.c_int),
                ("nseqthresh", C.c_int), ("alenthresh", C.c_int), ("abc", C.POINTER(Alphabet)), ("gpu", C.c_void_p)]


class RankList(C.Structure):
    _fields_ = [("ha", C.POINTER(Hist)), ("ht", C.POINTER(Hist)), ("hb", C.POINTER(Hist)),
                ("survfit", C.POINTER(C.c_double))]


class Hit(C.Structure):
    _fields_ = [("i", C.c_int64), ("j", C.c_int64), ("sc", C.c_double), ("Eval", C.c_double), ("pval", C.c_double),
                ("nsubs", C.c_int64), ("power", C.c_double), ("bptype", C.c_int), ("is_compatible", C.c_int)]


class HitList(C.Structure):
    _fields_ = [("nhit", C.c_int), ("srthit", C.c_void_p), ("hit", C.POINTER(Hit)), ("Nt", C.c_int64),
                ("Nb", C.c_int64)]


class Thresh(C.Structure):
    _fields_ = [("type", C.c_int), ("val", C.c_double), ("sc_bp", C.c_double), ("sc_nbp", C.c_double)]


class Rand(C.Structure):
    _fields_ = [("seed", C.c_uint64)]


class Data(C.Structure):
    _fields_ = [("r", C.POINTER(Rand)), ("samplesize", C.c_int), ("ranklist_null", C.POINTER(RankList)),
                ("ranklist_aux", C.POINTER(RankList)), ("mi", C.POINTER(Mutual)), ("thresh", C.POINTER(Thresh)),
                ("statsmethod", C.c_int), ("covmethod", C.c_int), ("mode", C.c_int), ("covtype", C.c_int),
                ("nseq", C.c_int), ("expBP", C.c_double), ("bmin", C.c_double), ("w", C.c_double),
                ("fracfit", C.c_double), ("pmass", C.c_double), ("doexpfit", C.c_int), ("tau", C.c_double),
                ("mu", C.c_double), ("lambda_", C.c_double), ("allowpair", C.POINTER(DMatrix)), ("tol", C.c_double),
                ("verbose", C.c_int), ("errbuf", C.c_char_p)]


GIVSS, RANSS = 0, 2


def setup_lib(path):
    lib = C.CDLL(path)
    lib.corr_Create.restype = C.POINTER(Mutual)
    lib.corr_Create.argtypes = [C.c_int64, C.c_int64, C.c_int, C.c_int, C.c_int, C.POINTER(Alphabet), C.c_int]
    lib.corr_Destroy.argtypes = [C.POINTER(Mutual)]
    lib.corr_Reuse.argtypes = [C.POINTER(Mutual), C.c_int, C.c_int, C.c_int]
    lib.cov_Calculate.argtypes = [C.POINTER(Data), C.POINTER(Msa), C.POINTER(C.POINTER(RankList)),
                                  C.POINTER(C.POINTER(HitList)), C.c_void_p, C.c_int]
    lib.corr_Probs.argtypes = [C.c_void_p, C.POINTER(Msa), C.c_void_p, C.c_void_p, C.POINTER(Mutual), C.c_int,
                               C.c_double, C.c_int, C.c_char_p]
    lib.corr_CalculateGT.argtypes = [C.c_int, C.POINTER(Data)]
    lib.corr_CalculateCOVCorrected.argtypes = [C.c_int, C.POINTER(Data), C.c_int]
    lib.cov_CreateRankList.restype = C.POINTER(RankList)
    lib.cov_CreateRankList.argtypes = [C.c_double, C.c_double, C.c_double]
    lib.cov_GrowRankList.argtypes = [C.POINTER(C.POINTER(RankList)), C.c_double, C.c_double]
    lib.cov_ranklist_Bin2Bin.argtypes = [C.c_int, C.POINTER(Hist), C.POINTER(Hist), C.POINTER(C.c_int)]
    lib.cov_FreeRankList.argtypes = [C.POINTER(RankList)]
    lib.cov_FreeHitList.argtypes = [C.POINTER(HitList)]
    return lib


class MsaHolder:
    def __init__(self, ax, wgt, abc):
        N, L = ax.shape
        self.rows = [np.concatenate([[255], ax[s], [255]]).astype(np.uint8) for s in range(N)]
        self.ptrs = (C.POINTER(C.c_uint8) * N)(*[r.ctypes.data_as(C.POINTER(C.c_uint8)) for r in self.rows])
        self.w = np.ascontiguousarray(wgt, dtype=np.float64)
        self.msa = Msa(self.ptrs, self.w.ctypes.data_as(C.POINTER(C.c_double)), N, L, C.pointer(abc))


def null_add(lib, rl, cum):
    """null_add2cumranklist, src/R-scape.c:1564-1612."""
    h = rl.contents.ha.contents
    if not cum:
        cum = lib.cov_CreateRankList(h.bmax, h.bmin, h.w)
        c = cum.contents.ha.contents
        c.n, c.xmin, c.xmax, c.imin, c.imax = h.n, h.xmin, h.xmax, h.imin, h.imax
    else:
        lib.cov_GrowRankList(C.byref(cum), h.bmax, h.bmin)
        c = cum.contents.ha.contents
        c.n += h.n
        c.xmin, c.xmax = min(c.xmin, h.xmin), max(c.xmax, h.xmax)
        c.imin, c.imax = min(c.imin, h.imin), max(c.imax, h.imax)
    c = cum.contents.ha.contents
    for b in range(h.imin, h.imax + 1):
        cb = C.c_int()
        lib.cov_ranklist_Bin2Bin(b, rl.contents.ha, cum.contents.ha, C.byref(cb))
        if cb.value < c.nb:
            c.obs[cb.value] += h.obs[b]
            c.Nc += h.obs[b]
            c.No += h.obs[b]
    return cum


@pytest.mark.parametrize("covtype", ["GTp", "MIp", "RAFp"])
def test_dropin_rscape_flow(covgpu, oracle, covtype):
    lib = setup_lib(covgpu.LIBPATH)
    N, L, ns = 160, 90, 6
    s = covgpu.Synth(N, L, 1.5, 18, 2, 9, 9, 0.08, seed=21, tree_kind=1)
    w = covgpu.weights_pb(s.ax)
    code = covgpu.covtype_code(covtype)
    abc = Alphabet(1, 4, 18)
    mi = lib.corr_Create(L, N, 0, 8, 50, C.byref(abc), 3)
    errbuf = C.create_string_buffer(256)
    th = Thresh(0, 0.05, 0.0, 0.0)
    rnd = Rand(42)
    data = Data(C.pointer(rnd), 3, None, None, mi, C.pointer(th), 1, 0, RANSS, code, N, -1.0, -10.0, 0.05, 1.0,
                0.0005, 0, 0.0, 0.0, 0.0, None, 1e-6, 0, C.cast(errbuf, C.c_char_p))
    T = oracle.TreeArrays(s.parent, s.left, s.right, s.ld, s.rd)
    cum = None
    for k in range(ns):
        nm = MsaHolder(oracle.null_msa(s.ax, T, 42, k), w, abc)
        if k == 0:   # calculate_width_histo
            lib.corr_Reuse(mi, 1, code, 3)
            assert lib.cov_Calculate(C.byref(data), C.byref(nm.msa), None, None, None, 0) == 0, errbuf.value
            m = mi.contents
            data.w = min(0.05, (m.maxCOV - max(-10.0, m.minCOV)) / 400)
        lib.corr_Reuse(mi, 1, code, 3)
        rl = C.POINTER(RankList)()
        assert lib.cov_Calculate(C.byref(data), C.byref(nm.msa), C.byref(rl), None, None, 1) == 0, errbuf.value
        cum = null_add(lib, rl, cum)
        lib.cov_FreeRankList(rl)
    data.mode = GIVSS
    data.ranklist_null = cum
    real = MsaHolder(s.ax, w, abc)
    lib.corr_Reuse(mi, 0, code, 3)
    rl = C.POINTER(RankList)()
    hl = C.POINTER(HitList)()
    assert lib.cov_Calculate(C.byref(data), C.byref(real.msa), C.byref(rl), C.byref(hl), None, 1) == 0, errbuf.value
    got = sorted((hl.contents.hit[k].i, hl.contents.hit[k].j) for k in range(hl.contents.nhit))
    ref = oracle.rscape(s.ax, w, T, covtype=covtype, nshuffle=ns)
    exp = sorted((i, j) for (i, j, sc, E, p) in ref["hits"])
    assert got == exp
    assert abs(data.w - ref["w"]) <= 1e-6 * ref["w"]
    ev = {(hl.contents.hit[k].i, hl.contents.hit[k].j): hl.contents.hit[k].Eval for k in range(hl.contents.nhit)}
    for (i, j, sc, E, p) in ref["hits"]:
        assert abs(ev[(i, j)] - E) <= 1e-5 * E
    # mi->Eval holds every pair's E-value, mi->COV the corrected scores
    Ev = np.ctypeslib.as_array(mi.contents.Eval.contents.mx[0], shape=(L * L,)).reshape(L, L)
    assert np.all(Ev[np.triu_indices(L, 1)] > 0)
    lib.cov_FreeHitList(hl)
    lib.cov_FreeRankList(rl)
    lib.cov_FreeRankList(cum)
    lib.corr_Destroy(mi)


def test_dropin_probs_and_statistic(covgpu, oracle):
    lib = setup_lib(covgpu.LIBPATH)
    N, L = 70, 55
    s = covgpu.Synth(N, L, 1.5, 9, 1, 9, 9, 0.08, seed=4, tree_kind=1)
    w = covgpu.weights_pb(s.ax)
    abc = Alphabet(1, 4, 18)
    mi = lib.corr_Create(L, N, 0, 8, 50, C.byref(abc), 3)
    errbuf = C.create_string_buffer(256)
    m = MsaHolder(s.ax, w, abc)
    assert lib.corr_Probs(None, C.byref(m.msa), None, None, mi, 0, 1e-6, 0, errbuf) == 0, errbuf.value
    opp, one, ong, opm, ops = oracle.probs(s.ax, w)
    pm = np.ctypeslib.as_array(mi.contents.pm[0], shape=(L * 4,)).reshape(L, 4)
    ne = np.ctypeslib.as_array(mi.contents.nseff[0], shape=(L * L,)).reshape(L, L)
    iu = np.triu_indices(L, 1)
    assert np.allclose(pm, opm, rtol=1e-6)
    assert np.allclose(ne[iu], one[iu], rtol=1e-6)
    th = Thresh(0, 0.05, 0.0, 0.0)
    data = Data(None, 3, None, None, mi, C.pointer(th), 1, 0, GIVSS, 4, N, -1.0, -10.0, 0.05, 1.0, 0.0005, 0, 0.0,
                0.0, 0.0, None, 1e-6, 0, C.cast(errbuf, C.c_char_p))
    assert lib.corr_CalculateGT(3, C.byref(data)) == 0
    assert lib.corr_CalculateCOVCorrected(0, C.byref(data), 0) == 0
    cov = np.ctypeslib.as_array(mi.contents.COV.contents.mx[0], shape=(L * L,)).reshape(L, L)
    ref, (rmin, rmax) = oracle.cov_calculate("GTp", s.ax, w)
    raw, _ = oracle.cov_calculate("GT", s.ax, w)
    assert np.all(np.abs(cov[iu] - ref[iu]) <= 1e-5 * np.abs(ref[iu]) + 1e-6 * np.abs(raw[iu]).max())
    assert mi.contents.type == 4
    assert abs(mi.contents.maxCOV - rmax) <= 1e-5 * abs(rmax)
    lib.corr_Destroy(mi)
