"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle restates R-scape's covariation path on the CPU in FP64 (see
rscape_oracle.h).  Only the tests, the smoke check and the CPU-baseline leg of
the benchmark load it; the GPU library never does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")

CHI, GT, MI, MIr, MIg, OMES, RAF, RAFS, CCF = 0, 3, 6, 9, 12, 15, 18, 21, 24
C16, C2, CWC, CSELECT = 0, 1, 2, 3
APC, ASC = 0, 1
COVTYPES = {"CHI": 0, "GT": 3, "MI": 6, "MIr": 9, "MIg": 12, "OMES": 15, "RAF": 18, "RAFS": 21, "CCF": 24}


def covtype_code(name):
    """'GTp' -> 4, 'MIa' -> 8, 'RAF' -> 18 (COVTYPE numbering)."""
    if name.endswith("p") and name[:-1] in COVTYPES:
        return COVTYPES[name[:-1]] + 1
    if name.endswith("a") and name[:-1] in COVTYPES:
        return COVTYPES[name[:-1]] + 2
    return COVTYPES[name]


class Tree(C.Structure):
    _fields_ = [("N", C.c_int), ("parent", C.POINTER(C.c_int)), ("left", C.POINTER(C.c_int)),
                ("right", C.POINTER(C.c_int)), ("ld", C.POINTER(C.c_double)), ("rd", C.POINTER(C.c_double))]


class Params(C.Structure):
    _fields_ = [("covtype", C.c_int), ("covclass", C.c_int), ("nseqthresh", C.c_int), ("alenthresh", C.c_int),
                ("nshuffle", C.c_int), ("thresh", C.c_double), ("bmin", C.c_double), ("w0", C.c_double),
                ("hpts", C.c_int), ("pmass", C.c_double), ("fracfit", C.c_double), ("doexpfit", C.c_int),
                ("tol", C.c_double), ("seed", C.c_uint64), ("allow", C.c_double * 16),
                ("samplesize", C.c_int), ("ncnt", C.c_int), ("cnt_i", C.c_void_p), ("cnt_j", C.c_void_p),
                ("cnt_type", C.c_void_p), ("mind", C.c_int), ("msa2pdb", C.c_void_p), ("expBP", C.c_double)]


class Result(C.Structure):
    _fields_ = [("nshuffle", C.c_int), ("w", C.c_double), ("null_minCOV", C.c_double), ("null_maxCOV", C.c_double),
                ("minCOV", C.c_double), ("maxCOV", C.c_double), ("pmass_used", C.c_double), ("newmass", C.c_double),
                ("mu", C.c_double), ("lambda_", C.c_double), ("tau", C.c_double), ("fit_ok", C.c_int),
                ("sc_thresh", C.c_double), ("Nt", C.c_uint64), ("nhit", C.c_int),
                ("h_bmin", C.c_double), ("h_w", C.c_double), ("h_nb", C.c_int), ("h_imin", C.c_int),
                ("h_imax", C.c_int), ("h_cmin", C.c_int), ("h_n", C.c_uint64), ("h_Nc", C.c_uint64),
                ("h_No", C.c_uint64), ("h_xmin", C.c_double), ("h_xmax", C.c_double), ("h_phi", C.c_double),
                ("sc_nbp", C.c_double), ("Nb", C.c_uint64)]


def build(force=False):
    so = os.path.join(_HERE, "librscape_oracle.so")
    src = os.path.join(_HERE, "rscape_oracle.c")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return so


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(build())
        L.orc_philox4x32.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_weights_pb.argtypes = [u8p, C.c_int, C.c_int, f64p]
        L.orc_weights_gsc.argtypes = [u8p, C.c_int, C.c_int, f64p]
        L.orc_gapfilter.argtypes = [u8p, f64p, C.c_int, C.c_int, C.c_double, i32p]
        L.orc_probs.argtypes = [u8p, f64p, C.c_int, C.c_int, C.c_double, f64p, f64p, f64p, f64p, f64p]
        L.orc_stat.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, f64p, f64p, f64p, f64p,
                               f64p, f64p, f64p]
        L.orc_raf.argtypes = [u8p, C.c_int, C.c_int, f64p, f64p, f64p]
        L.orc_rafs.argtypes = [u8p, C.c_int, C.c_int, f64p, f64p, f64p]
        L.orc_ccf.argtypes = [C.c_int, f64p, f64p, f64p, f64p]
        L.orc_cov_corrected.argtypes = [C.c_int, C.c_int, f64p, f64p]
        L.orc_cov_calculate.argtypes = [C.c_int, C.c_int, u8p, f64p, C.c_int, C.c_int, C.c_int, C.c_int, f64p,
                                        C.c_double, f64p, f64p]
        L.orc_feistel_perm.argtypes = [C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32)]
        L.orc_feistel_perm.restype = C.c_uint32
        L.orc_fitch.argtypes = [u8p, C.c_int, C.c_int, C.POINTER(Tree), C.c_uint64, C.c_uint32, u8p]
        L.orc_null_msa.argtypes = [u8p, C.c_int, C.c_int, C.POINTER(Tree), C.c_uint64, C.c_uint32, u8p]
        L.orc_params_default.argtypes = [C.POINTER(Params)]
        L.orc_rscape.argtypes = [C.POINTER(Params), u8p, f64p, C.c_int, C.c_int, C.POINTER(Tree),
                                 C.c_void_p, C.c_void_p, u64p, C.c_int,
                                 i32p, i32p, f64p, f64p, f64p, C.c_int, C.POINTER(Result)]
        L.orc_faithful_rows.argtypes = [u8p, f64p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.POINTER(C.c_double)]
        L.orc_faithful_rows.restype = C.c_double
        L.orc_faithful_raf.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.orc_faithful_raf.restype = C.c_double
        L.orc_sim_conditionals.argtypes = [f64p, C.c_int, C.c_double, f64p]
        L.orc_substitutions.argtypes = [u8p, C.c_int, C.c_int, C.POINTER(Tree), C.c_uint64, C.c_uint32, C.c_int,
                                        i32p, i32p, i32p]
        L.orc_power_step.argtypes = [C.c_double, C.c_int, f64p, f64p]
        L.orc_power_step.restype = C.c_double
        L.orc_sim_cdf.argtypes = [f64p, C.c_int, C.c_int, u64p]
        L.orc_sim_cdf.restype = None
        L.orc_simulate.argtypes = [C.POINTER(Tree), C.c_int, C.c_int, i32p, u64p, u64p, u64p, u64p, C.c_void_p,
                                   C.c_double, C.c_double, C.c_uint64, C.c_uint32, u8p]
        f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
        L.orc_raf_pairs.argtypes = [u8p, C.c_int, C.c_int, f64p, C.c_int, i32p, i32p, f64p]
        L.orc_raf_pairs.restype = None
        L.orc_features.argtypes = [u8p, C.c_int, C.c_int, f64p, C.c_double, f64p]
        L.orc_features.restype = None
        L.orc_mlp_forward.argtypes = [f32p, f32p, f32p, C.c_int, f64p]
        L.orc_mlp_forward.restype = None
        L.orc_mlp_grad.argtypes = [f32p, f32p, f32p, f32p, C.c_int, f64p]
        L.orc_mlp_grad.restype = C.c_double
        L.orc_raf_counts.argtypes = [u8p, C.c_int, C.c_int, f64p, f64p, f64p]
        L.orc_rscape_multi.argtypes = [C.POINTER(Params), C.c_int, C.c_void_p, u8p, f64p, C.c_int, C.c_int,
                                       C.POINTER(Tree), C.c_void_p, C.c_void_p, u64p, C.c_int, i32p, i32p, f64p, f64p,
                                       f64p, C.c_int, C.c_void_p]
        for f in ("orc_agg_fisher", "orc_agg_sidak"):
            getattr(L, f).argtypes = [C.c_int, f64p]
            getattr(L, f).restype = C.c_double
        L.orc_agg_weighted.argtypes = [C.c_int, f64p, f64p]
        L.orc_agg_weighted.restype = C.c_double
        for f in ("orc_agg_weights_lancaster", "orc_agg_weights_wfisher"):
            getattr(L, f).argtypes = [C.c_int, f64p, f64p]
            getattr(L, f).restype = None
        _LIB = L
    return _LIB


def default_allow():
    a = np.zeros(16)
    for x, y in ((0, 3), (3, 0), (1, 2), (2, 1), (2, 3), (3, 2)):
        a[x * 4 + y] = 1.0
    return a


def philox(key, ctr):
    k = (C.c_uint32 * 2)(*key)
    c = (C.c_uint32 * 4)(*ctr)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32(k, c, o)
    return list(o)


def weights_pb(ax):
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    w = np.zeros(ax.shape[0])
    lib().orc_weights_pb(ax, ax.shape[0], ax.shape[1], w)
    return w


def weights_gsc(ax):
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    w = np.zeros(ax.shape[0])
    lib().orc_weights_gsc(ax, ax.shape[0], ax.shape[1], w)
    return w


def gapfilter(ax, wgt=None, gapthresh=0.75):
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    N, L = ax.shape
    wgt = np.ones(N) if wgt is None else np.ascontiguousarray(wgt, dtype=np.float64)
    use = np.zeros(L, dtype=np.int32)
    lib().orc_gapfilter(ax, wgt, N, L, gapthresh, use)
    return use.astype(bool)


def probs(ax, wgt, tol=1e-6):
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    wgt = np.ascontiguousarray(wgt, dtype=np.float64)
    N, L = ax.shape
    pp = np.zeros(L * L * 16)
    nseff = np.zeros(L * L)
    ngap = np.zeros(L * L)
    pm = np.zeros(L * 4)
    ps = np.zeros(L * 5)
    st = lib().orc_probs(ax, wgt, N, L, tol, pp, nseff, ngap, pm, ps)
    if st:
        raise RuntimeError("orc_probs failed %d" % st)
    return (pp.reshape(L, L, 16), nseff.reshape(L, L), ngap.reshape(L, L), pm.reshape(L, 4), ps.reshape(L, 5))


def cov_calculate(covtype, ax, wgt, covclass=CSELECT, nseqthresh=8, alenthresh=50, allow=None, tol=1e-6):
    """COV (L x L) and (minCOV, maxCOV) for a covtype name ('GTp') or code."""
    if isinstance(covtype, str):
        covtype = covtype_code(covtype)
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    wgt = np.ascontiguousarray(wgt, dtype=np.float64)
    N, L = ax.shape
    allow = default_allow() if allow is None else np.ascontiguousarray(allow, dtype=np.float64)
    COV = np.zeros(L * L)
    mm = np.zeros(2)
    st = lib().orc_cov_calculate(covtype, covclass, ax, wgt, N, L, nseqthresh, alenthresh, allow, tol, COV, mm)
    if st:
        raise RuntimeError("orc_cov_calculate failed %d" % st)
    return COV.reshape(L, L), (mm[0], mm[1])


class TreeArrays:
    """Keeps the numpy arrays of an Easel-convention tree alive for ctypes."""

    def __init__(self, parent, left, right, ld, rd):
        self.parent = np.ascontiguousarray(parent, dtype=np.int32)
        self.left = np.ascontiguousarray(left, dtype=np.int32)
        self.right = np.ascontiguousarray(right, dtype=np.int32)
        self.ld = np.ascontiguousarray(ld, dtype=np.float64)
        self.rd = np.ascontiguousarray(rd, dtype=np.float64)
        self.N = len(self.parent) + 1
        ip = C.POINTER(C.c_int)
        dp = C.POINTER(C.c_double)
        self.ct = Tree(self.N, self.parent.ctypes.data_as(ip), self.left.ctypes.data_as(ip),
                       self.right.ctypes.data_as(ip), self.ld.ctypes.data_as(dp), self.rd.ctypes.data_as(dp))


def feistel_perm(t, L, rk):
    arr = (C.c_uint32 * 6)(*rk)
    return lib().orc_feistel_perm(t, L, arr)


def fitch(ax, tree, seed, null_id):
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    N, L = ax.shape
    out = np.zeros((2 * N - 1) * L, dtype=np.uint8)
    st = lib().orc_fitch(ax, N, L, C.byref(tree.ct), seed, null_id, out)
    if st:
        raise RuntimeError("orc_fitch failed")
    return out.reshape(2 * N - 1, L)


def null_msa(ax, tree, seed, null_id):
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    N, L = ax.shape
    out = np.zeros(N * L, dtype=np.uint8)
    st = lib().orc_null_msa(ax, N, L, C.byref(tree.ct), seed, null_id, out)
    if st:
        raise RuntimeError("orc_null_msa failed")
    return out.reshape(N, L)


def substitutions(ax, tree, seed, null_id, includegaps=False):
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    N, L = ax.shape
    ns = np.zeros(L, dtype=np.int32)
    nd = np.zeros(L * L, dtype=np.int32)
    nj = np.zeros(L * L, dtype=np.int32)
    st = lib().orc_substitutions(ax, N, L, C.byref(tree.ct), seed, null_id, 1 if includegaps else 0, ns, nd, nj)
    if st:
        raise RuntimeError("orc_substitutions failed (%d)" % st)
    return ns, nd.reshape(L, L), nj.reshape(L, L)


def power_step(n, subs, prob):
    subs = np.ascontiguousarray(subs, dtype=np.float64)
    prob = np.ascontiguousarray(prob, dtype=np.float64)
    return lib().orc_power_step(float(n), len(subs), subs, prob)


def sim_conditionals(Q, rt):
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    n = Q.shape[0]
    P = np.zeros((n, n))
    st = lib().orc_sim_conditionals(Q, n, float(rt), P)
    if st:
        raise RuntimeError("orc_sim_conditionals failed (%d)" % st)
    return P


def sim_cdf(P):
    P = np.ascontiguousarray(P, dtype=np.float64)
    n = P.shape[-1]
    rows = P.size // n
    out = np.zeros(P.size, dtype=np.uint64)
    lib().orc_sim_cdf(P, n, rows, out)
    return out.reshape(P.shape)


def simulate(tree, L, ct, P4, P16, pi4, pi16, root, gap_rate, gap_mean, seed, rep):
    """One simulated alignment [N][L] from per-branch P tables (branch 2v+side)."""
    N = tree.N
    C4 = sim_cdf(np.asarray(P4).reshape(-1, 4, 4))
    C16 = sim_cdf(np.asarray(P16).reshape(-1, 16, 16))
    R4 = sim_cdf(np.asarray(pi4, dtype=np.float64).reshape(1, 4))
    R16 = sim_cdf(np.asarray(pi16, dtype=np.float64).reshape(1, 16))
    ctv = np.ascontiguousarray(ct, dtype=np.int32)
    out = np.zeros(N * L, dtype=np.uint8)
    rt = None if root is None else np.ascontiguousarray(root, dtype=np.uint8)
    st = lib().orc_simulate(C.byref(tree.ct), N, L, ctv, np.ascontiguousarray(C4), np.ascontiguousarray(C16),
                            np.ascontiguousarray(R4), np.ascontiguousarray(R16),
                            None if rt is None else rt.ctypes.data, float(gap_rate), float(gap_mean), seed, rep,
                            out)
    if st:
        raise RuntimeError("orc_simulate failed (%d)" % st)
    return out.reshape(N, L)


SAMPLE_CONTACTS, SAMPLE_BP, SAMPLE_WC, SAMPLE_ALL = 0, 1, 2, 3
WWc, STACKED, CONTACT, BPNONE = 0, 32, 33, 34


def params(**kw):
    """orc_params_t with R-scape's defaults, overridden by kw.  contacts =
    [(i, j, bptype), ...] (1-based alignment positions) and msa2pdb (an
    int array over the columns, -1 where a column has no PDB position) are
    kept alive on the returned object."""
    p = Params()
    lib().orc_params_default(C.byref(p))
    keep = []
    for k, v in kw.items():
        if k == "covtype" and isinstance(v, str):
            v = covtype_code(v)
        if k == "allow":
            for i in range(16):
                p.allow[i] = float(v[i])
            continue
        if k == "contacts":
            c = np.asarray(v, dtype=np.int64).reshape(-1, 3)
            ci, cj = np.ascontiguousarray(c[:, 0]), np.ascontiguousarray(c[:, 1])
            ct = np.ascontiguousarray(c[:, 2].astype(np.int32))
            keep += [ci, cj, ct]
            p.ncnt = len(c)
            p.cnt_i, p.cnt_j, p.cnt_type = ci.ctypes.data, cj.ctypes.data, ct.ctypes.data
            continue
        if k == "msa2pdb":
            m = np.ascontiguousarray(v, dtype=np.int32)
            keep.append(m)
            p.msa2pdb = m.ctypes.data
            continue
        setattr(p, k, v)
    p._keep = keep
    return p


def rscape(ax, wgt, tree, want_matrices=False, hit_cap=1 << 20, **kw):
    """Whole per-alignment path: nulls, fit, E-values.  Returns a dict."""
    p = params(**kw)
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    wgt = np.ascontiguousarray(wgt, dtype=np.float64)
    N, L = ax.shape
    COV = np.zeros(L * L) if want_matrices else None
    Ev = np.zeros(L * L) if want_matrices else None
    cap = 1 << 16
    obs = np.zeros(cap, dtype=np.uint64)
    hi = np.zeros(hit_cap, dtype=np.int32)
    hj = np.zeros(hit_cap, dtype=np.int32)
    hs = np.zeros(hit_cap)
    he = np.zeros(hit_cap)
    hp = np.zeros(hit_cap)
    res = Result()
    st = lib().orc_rscape(C.byref(p), ax, wgt, N, L, C.byref(tree.ct),
                          COV.ctypes.data if COV is not None else None,
                          Ev.ctypes.data if Ev is not None else None,
                          obs, cap, hi, hj, hs, he, hp, hit_cap, C.byref(res))
    if st:
        raise RuntimeError("orc_rscape failed %d" % st)
    n = min(res.nhit, hit_cap)
    out = {f[0]: getattr(res, f[0]) for f in Result._fields_}
    out["null_obs"] = obs[:res.h_nb].copy()
    out["hits"] = list(zip(hi[:n].tolist(), hj[:n].tolist(), hs[:n].tolist(), he[:n].tolist(), hp[:n].tolist()))
    if want_matrices:
        out["COV"] = COV.reshape(L, L)
        out["Eval"] = Ev.reshape(L, L)
    return out


def rscape_multi(ax, wgt, tree, covtypes, hit_cap=1 << 20, **kw):
    """rscape() for several statistics that share the null alignments (each
    alignment's probabilities formed once); a list of dicts, one per
    statistic, as rscape() returns."""
    p = params(**kw)
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    wgt = np.ascontiguousarray(wgt, dtype=np.float64)
    N, L = ax.shape
    nt = len(covtypes)
    codes = np.array([covtype_code(t) for t in covtypes], dtype=np.int32)
    cap = 1 << 16
    obs = np.zeros(nt * cap, dtype=np.uint64)
    hi = np.zeros(nt * hit_cap, dtype=np.int32)
    hj = np.zeros(nt * hit_cap, dtype=np.int32)
    hs = np.zeros(nt * hit_cap)
    he = np.zeros(nt * hit_cap)
    hp = np.zeros(nt * hit_cap)
    res = (Result * nt)()
    st = lib().orc_rscape_multi(C.byref(p), nt, codes.ctypes.data, ax, wgt, N, L, C.byref(tree.ct), None, None,
                                obs, cap, hi, hj, hs, he, hp, hit_cap, res)
    if st:
        raise RuntimeError("orc_rscape_multi failed %d" % st)
    out = []
    for t in range(nt):
        r = res[t]
        n = min(r.nhit, hit_cap)
        o = t * hit_cap
        d = {f[0]: getattr(r, f[0]) for f in Result._fields_}
        d["null_obs"] = obs[t * cap:t * cap + r.h_nb].copy()
        d["hits"] = list(zip(hi[o:o + n].tolist(), hj[o:o + n].tolist(), hs[o:o + n].tolist(),
                             he[o:o + n].tolist(), hp[o:o + n].tolist()))
        out.append(d)
    return out


def faithful_rows(ax, wgt, i0, i1, nthreads=0):
    """Times nothing itself: runs the reference loop nest for rows [i0,i1)."""
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    wgt = np.ascontiguousarray(wgt, dtype=np.float64)
    N, L = ax.shape
    cs = C.c_double()
    npairs = lib().orc_faithful_rows(ax, wgt, N, L, i0, i1, nthreads, C.byref(cs))
    return int(npairs), cs.value


def faithful_raf(ax, npairs, nthreads=0):
    """Runs corr_CalculateRAF's O(N^2) loop for the first npairs pairs."""
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    N, L = ax.shape
    cs = C.c_double()
    n = lib().orc_faithful_raf(ax, N, L, npairs, nthreads, C.byref(cs))
    return int(n), cs.value


def features(ax, wgt, tree_len):
    """The 64 learned-null features of ax [N][L] with weights wgt, in FP64."""
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    N, L = ax.shape
    f = np.zeros(64)
    lib().orc_features(ax, N, L, np.ascontiguousarray(wgt, dtype=np.float64), float(tree_len), f)
    return f


def mlp_forward(params, nrm, X):
    """De-standardised outputs [n][3] of the learned-null network in FP64."""
    X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, 64)
    Y = np.zeros((X.shape[0], 3))
    lib().orc_mlp_forward(np.ascontiguousarray(params, dtype=np.float32), np.ascontiguousarray(nrm, dtype=np.float32),
                          X, X.shape[0], Y)
    return Y


def mlp_grad(params, nrm, X, T):
    """(loss, gradient[148995]) of the network's mean squared error in FP64."""
    X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, 64)
    T = np.ascontiguousarray(T, dtype=np.float32).reshape(-1, 3)
    g = np.zeros(148995)
    loss = lib().orc_mlp_grad(np.ascontiguousarray(params, dtype=np.float32),
                              np.ascontiguousarray(nrm, dtype=np.float32), X, T, X.shape[0], g)
    return loss, g


def raf_pairs(ax, pairs, allow=None):
    """RAF of the listed (i, j) pairs with the reference's O(N^2) loop."""
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    N, L = ax.shape
    pi = np.ascontiguousarray([p[0] for p in pairs], dtype=np.int32)
    pj = np.ascontiguousarray([p[1] for p in pairs], dtype=np.int32)
    out = np.zeros(len(pairs))
    allow = default_allow() if allow is None else np.ascontiguousarray(allow, dtype=np.float64)
    lib().orc_raf_pairs(ax, N, L, allow, len(pairs), pi, pj, out)
    return out


AGG_FISHER, AGG_LANCASTER, AGG_WFISHER, AGG_SIDAK = 0, 1, 2, 3


def agg_weights(method, aux):
    """extract_rm_weights_lancaster (1 + substitutions) or
    extract_rm_weights_wfisher ((0.01 + power), scaled to sum 2n) of one
    helix (src/aggregate.c:375-488)."""
    aux = np.ascontiguousarray(aux, dtype=np.float64)
    w = np.zeros(len(aux))
    if method == AGG_LANCASTER:
        lib().orc_agg_weights_lancaster(len(aux), aux, w)
    else:
        lib().orc_agg_weights_wfisher(len(aux), aux, w)
    return w


def agg_pvalue(method, pvals, aux=None):
    """The aggregated p-value of one helix (agg_FISHER, agg_LANCASTER,
    agg_WFISHER, agg_SIDAK of src/aggregate.c:146-322); aux holds the
    pairs' substitution counts (Lancaster) or powers (weighted Fisher)."""
    p = np.ascontiguousarray(pvals, dtype=np.float64)
    n = len(p)
    if method == AGG_FISHER:
        return lib().orc_agg_fisher(n, p)
    if method == AGG_SIDAK:
        return lib().orc_agg_sidak(n, p)
    return lib().orc_agg_weighted(n, p, agg_weights(method, aux))
