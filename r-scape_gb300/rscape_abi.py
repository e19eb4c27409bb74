"""ctypes binding of the reference-named entry points (include/rscape_cov.h):
the layout shims of struct mutual_s, struct data_s, ESL_MSA, ESL_DMATRIX,
ESL_HISTOGRAM, RANKLIST and HITLIST, and R-scape's calling sequence for one
alignment (null_rscape and rscape_for_msa, src/R-scape.c:1564-1724, 2502),
as a caller of the drop-in library would write them.  Used by the tests and
the benchmark; the product is the C library itself."""
import ctypes as C

import numpy as np


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
                ("nseqthresh", C.c_int), ("alenthresh", C.c_int), ("abc", C.POINTER(Alphabet)), ("gpu", C.c_void_p),
                ("device_resident", C.c_int)]


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


class Cnt(C.Structure):
    _fields_ = [("i", C.c_int64), ("j", C.c_int64), ("bptype", C.c_int)]


class Clist(C.Structure):
    _fields_ = [("ncnt", C.c_int), ("mind", C.c_int), ("cnt", C.POINTER(Cnt))]


def make_clist(contacts, mind=0):
    """A CLIST of contacts [(i, j, bptype), ...] (1-based alignment
    positions, i < j), the contact array kept alive on the object."""
    arr = (Cnt * max(1, len(contacts)))(*[Cnt(int(i), int(j), int(t)) for (i, j, t) in contacts])
    cl = Clist(len(contacts), mind, arr)
    cl._arr = arr
    return cl


class Data(C.Structure):
    _fields_ = [("r", C.POINTER(Rand)), ("samplesize", C.c_int), ("ranklist_null", C.POINTER(RankList)),
                ("ranklist_aux", C.POINTER(RankList)), ("mi", C.POINTER(Mutual)), ("thresh", C.POINTER(Thresh)),
                ("statsmethod", C.c_int), ("covmethod", C.c_int), ("mode", C.c_int), ("covtype", C.c_int),
                ("nseq", C.c_int), ("expBP", C.c_double), ("bmin", C.c_double), ("w", C.c_double),
                ("fracfit", C.c_double), ("pmass", C.c_double), ("doexpfit", C.c_int), ("tau", C.c_double),
                ("mu", C.c_double), ("lambda_", C.c_double), ("allowpair", C.POINTER(DMatrix)), ("tol", C.c_double),
                ("verbose", C.c_int), ("errbuf", C.c_char_p), ("clist", C.POINTER(Clist)),
                ("msa2pdb", C.POINTER(C.c_int))]


GIVSS, RANSS = 0, 2
SAMPLE_CONTACTS, SAMPLE_BP, SAMPLE_WC, SAMPLE_ALL = 0, 1, 2, 3
WWc, STACKED, CONTACT, BPNONE = 0, 32, 33, 34


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
    lib.corr_SyncHost.argtypes = [C.POINTER(Mutual), C.c_char_p]
    return lib


class MsaHolder:
    def __init__(self, ax, wgt, abc):
        N, L = ax.shape
        self.rows = [np.concatenate([[255], ax[s], [255]]).astype(np.uint8) for s in range(N)]
        self.ptrs = (C.POINTER(C.c_uint8) * N)(*[r.ctypes.data_as(C.POINTER(C.c_uint8)) for r in self.rows])
        self.w = np.ascontiguousarray(wgt, dtype=np.float64)
        self.msa = Msa(self.ptrs, self.w.ctypes.data_as(C.POINTER(C.c_double)), N, L, C.pointer(abc))


def bin2bin(h, c, b):
    """cov_ranklist_Bin2Bin (src/covariation.c:2334-2362) for the bins b of
    histogram h into histogram c, in FP64 as the library computes it: the
    bins and whether each lies in [0, c.nb)."""
    x = h.w * np.asarray(b, dtype=np.float64) + h.bmin
    v = (x - c.bmin) / c.w
    t = np.trunc(v)
    r = t + np.where(np.abs(v - t) >= 0.5, np.sign(v), 0.0)   # C's round(): halves away from zero
    ok = np.isfinite(r) & (r >= 0) & (r < c.nb)
    return np.where(ok, r, -1).astype(np.int64), ok


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
    if h.imax < h.imin:
        return cum
    # the reference's loop over bins imin..imax, where only the non-empty
    # bins change the sum, mapped as cov_ranklist_Bin2Bin maps them
    # (src/covariation.c:2334-2362): x = w b + bmin, then C's round() of
    # (x - bmin') / w' (halves away from zero), all in FP64
    obs = np.ctypeslib.as_array(h.obs, shape=(h.nb,))
    cobs = np.ctypeslib.as_array(c.obs, shape=(c.nb,))
    b = np.flatnonzero(obs[h.imin:h.imax + 1]) + h.imin
    r, ok = bin2bin(h, c, b)
    add = obs[b[ok]]
    np.add.at(cobs, r[ok], add)
    n = int(add.sum())
    c.Nc += n
    c.No += n
    return cum


def rscape_flow(lib, mi, nulls, real, data, code, timing=None):
    """R-scape's per-alignment path through the reference-named entry points
    (src/R-scape.c:1614-1724, 2502): calculate_width_histo on the first null
    (:1281-1371), cov_Calculate in RANSS mode on every null merged into the
    cumulative null histogram, then cov_Calculate in GIVSS mode on the
    alignment.  nulls and real are MsaHolder objects; data is the caller's
    struct data_s.  With a dict for timing, the wall seconds of each step
    (corr_Reuse, the nulls' cov_Calculate, the merge, the alignment's
    cov_Calculate) are added to it.  Returns (ranklist, hitlist, cumulative
    null ranklist)."""
    import time

    def step(name, f, *a):
        t0 = time.perf_counter()
        r = f(*a)
        if timing is not None:
            timing[name] = timing.get(name, 0.0) + time.perf_counter() - t0
        return r

    data.mode = RANSS
    data.ranklist_null = None
    cum = None
    errbuf = data.errbuf
    for k, nm in enumerate(nulls):
        if k == 0:
            step("corr_Reuse", lib.corr_Reuse, mi, 1, code, 3)
            if step("cov_Calculate_nulls", lib.cov_Calculate, C.byref(data), C.byref(nm.msa), None, None, None, 0):
                raise RuntimeError(errbuf)
            m = mi.contents
            data.w = min(0.05, (m.maxCOV - max(-10.0, m.minCOV)) / 400)
        step("corr_Reuse", lib.corr_Reuse, mi, 1, code, 3)
        rl = C.POINTER(RankList)()
        if step("cov_Calculate_nulls", lib.cov_Calculate, C.byref(data), C.byref(nm.msa), C.byref(rl), None, None, 1):
            raise RuntimeError(errbuf)
        cum = step("null_merge", null_add, lib, rl, cum)
        lib.cov_FreeRankList(rl)
    data.mode = GIVSS
    data.ranklist_null = cum
    step("corr_Reuse", lib.corr_Reuse, mi, 0, code, 3)
    rl = C.POINTER(RankList)()
    hl = C.POINTER(HitList)()
    if step("cov_Calculate_alignment", lib.cov_Calculate, C.byref(data), C.byref(real.msa), C.byref(rl), C.byref(hl),
            None, 1):
        raise RuntimeError(errbuf)
    return rl, hl, cum
