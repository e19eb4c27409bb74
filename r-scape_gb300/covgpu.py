"""Python binding of libcovgpu.so (the GB300 covariation engine).

Thin ctypes layer over the C-ABI in include/covgpu.h.  There is no CPU path:
if the shared library cannot be loaded, or no CUDA device is present, the
calls raise.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "libcovgpu.so")
_LIB = None

u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

COVTYPES = {"CHI": 0, "GT": 3, "MI": 6, "MIr": 9, "MIg": 12, "OMES": 15, "RAF": 18, "RAFS": 21, "CCF": 24}
C16, C2, CWC, CSELECT = 0, 1, 2, 3
SIMT, TENSOR = 0, 1


def covtype_code(name):
    """'GTp' -> 4, 'MIa' -> 8, 'RAF' -> 18 (R-scape's COVTYPE numbering)."""
    if isinstance(name, int):
        return name
    if name.endswith("p") and name[:-1] in COVTYPES:
        return COVTYPES[name[:-1]] + 1
    if name.endswith("a") and name[:-1] in COVTYPES:
        return COVTYPES[name[:-1]] + 2
    return COVTYPES[name]


class Params(C.Structure):
    _fields_ = [("covclass", C.c_int), ("nseqthresh", C.c_int), ("alenthresh", C.c_int), ("nshuffle", C.c_int),
                ("thresh", C.c_double), ("bmin", C.c_double), ("w0", C.c_double), ("hpts", C.c_int),
                ("pmass", C.c_double), ("fracfit", C.c_double), ("doexpfit", C.c_int), ("tol", C.c_double),
                ("seed", C.c_uint64), ("allow", C.c_double * 16), ("counter", C.c_int),
                ("samplesize", C.c_int), ("ncnt", C.c_int), ("cnt_i", C.c_void_p), ("cnt_j", C.c_void_p),
                ("cnt_type", C.c_void_p), ("expBP", C.c_double)]


class Result(C.Structure):
    _fields_ = [("covtype", C.c_int), ("status", C.c_int), ("nshuffle", C.c_int), ("w", C.c_double),
                ("minCOV", C.c_double), ("maxCOV", C.c_double), ("null_minCOV", C.c_double),
                ("null_maxCOV", C.c_double), ("pmass", C.c_double), ("newmass", C.c_double), ("mu", C.c_double),
                ("lambda_", C.c_double), ("tau", C.c_double), ("sc_thresh", C.c_double), ("Nt", C.c_uint64),
                ("nhit", C.c_int), ("h_bmin", C.c_double), ("h_w", C.c_double), ("h_xmin", C.c_double),
                ("h_xmax", C.c_double), ("h_phi", C.c_double), ("h_nb", C.c_int), ("h_imin", C.c_int),
                ("h_imax", C.c_int), ("h_cmin", C.c_int), ("h_n", C.c_uint64), ("h_Nc", C.c_uint64),
                ("h_No", C.c_uint64), ("sc_nbp", C.c_double), ("Nb", C.c_uint64)]


class Hit(C.Structure):
    _fields_ = [("i", C.c_int), ("j", C.c_int), ("sc", C.c_double), ("E", C.c_double), ("pval", C.c_double)]


class Family(C.Structure):
    _fields_ = [("N", C.c_int), ("L", C.c_int), ("ax", C.c_void_p), ("wgt", C.c_void_p), ("parent", C.c_void_p),
                ("left", C.c_void_p), ("right", C.c_void_p)]


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError("libcovgpu.so is not built (run __graft_entry__.build())")
        L = C.CDLL(LIBPATH)
        vp = C.c_void_p
        L.covgpu_params_default.argtypes = [C.POINTER(Params)]
        L.covgpu_errmsg.argtypes = [vp]
        L.covgpu_errmsg.restype = C.c_char_p
        L.covgpu_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.covgpu_destroy.argtypes = [vp]
        L.covgpu_set_weights.argtypes = [vp, f64p]
        L.covgpu_set_alignment.argtypes = [vp, C.c_int, u8p]
        L.covgpu_get_alignment.argtypes = [vp, C.c_int, u8p]
        L.covgpu_set_tree.argtypes = [vp, i32p, i32p, i32p]
        L.covgpu_make_nulls.argtypes = [vp, C.c_uint64, C.c_int, C.c_int, C.c_int]
        L.covgpu_simulate.argtypes = [vp, f64p, f64p, f64p, f64p, f64p, f64p, i32p, vp, C.c_double, C.c_double,
                                      C.c_uint64, C.c_uint32, C.c_int, C.c_int]
        L.covgpu_sim_tables.argtypes = [vp, f64p, f64p]
        L.covgpu_weights_pb_dev.argtypes = [vp, C.c_int, C.c_int, f64p]
        L.covgpu_weights_gsc_dev.argtypes = [vp, C.c_int, C.c_int, f64p]
        L.covgpu_substitutions.argtypes = [vp, C.c_int, C.c_uint64, C.c_int, i32p, i32p, i32p]
        L.covgpu_power.argtypes = [vp, C.c_int] + [vp] * 9
        L.covgpu_gapfilter_dev.argtypes = [vp, C.c_int, vp, C.c_double, i32p]
        L.covgpu_synth_model.argtypes = [f64p, f64p, f64p, f64p]
        L.covgpu_score.argtypes = [vp, C.c_int, C.c_int, C.c_int, i32p, C.c_int, C.c_int, C.c_int, f64p, C.c_int,
                                   f64p]
        L.covgpu_get_cov.argtypes = [vp, C.c_int, C.c_int, f64p]
        L.covgpu_get_probs.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, vp]
        L.covgpu_rscape.argtypes = [vp, C.POINTER(Params), u8p, f64p, C.c_int, i32p, C.POINTER(Result),
                                    C.POINTER(Hit), C.c_int]
        L.covgpu_last_timing.argtypes = [vp, f64p, C.POINTER(C.c_int)]
        L.covgpu_flush_l2.argtypes = [vp]
        L.covgpu_rscape.argtypes = [vp, C.POINTER(Params), vp, vp, C.c_int, i32p, C.POINTER(Result),
                                    C.POINTER(Hit), C.c_int]
        L.covgpu_synth.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                   C.c_double, C.c_uint64, u8p, i32p, i32p, i32p, f64p, f64p, i32p]
        L.covgpu_synth2.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_double, C.c_double, C.c_uint64, u8p, i32p, i32p, i32p, f64p, f64p, i32p]
        L.covgpu_weights_pb.argtypes = [u8p, C.c_int, C.c_int, f64p]
        L.covgpu_gapfilter.argtypes = [u8p, f64p, C.c_int, C.c_int, C.c_double, i32p]
        L.covgpu_features.argtypes = [vp, C.c_int, C.c_double, f32p]
        L.covgpu_mlp_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_uint64]
        L.covgpu_mlp_destroy.argtypes = [vp]
        L.covgpu_mlp_errmsg.argtypes = [vp]
        L.covgpu_mlp_errmsg.restype = C.c_char_p
        L.covgpu_mlp_set_params.argtypes = [vp, f32p]
        L.covgpu_mlp_get_params.argtypes = [vp, f32p]
        L.covgpu_mlp_set_members.argtypes = [vp, vp, C.c_int]
        L.covgpu_mlp_set_norm.argtypes = [vp, f32p, f32p, f32p, f32p, vp, vp]
        L.covgpu_mlp_get_norm.argtypes = [vp, f32p, f32p, f32p, f32p, f32p, f32p]
        L.covgpu_mlp_in_range.argtypes = [vp, f32p]
        L.covgpu_mlp_forward.argtypes = [vp, f32p, C.c_int, f32p]
        L.covgpu_mlp_grad.argtypes = [vp, f32p, f32p, C.c_int, f32p, C.POINTER(C.c_float)]
        L.covgpu_mlp_train.argtypes = [vp, f32p, f32p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_uint64,
                                       f32p]
        L.covgpu_resize.argtypes = [vp, C.c_int, C.c_int]
        L.covgpu_autotune.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, f32p, C.POINTER(C.c_int)]
        L.covgpu_helices.argtypes = [i32p, C.c_int, C.c_int, C.POINTER(C.c_int), i32p, i32p, i32p]
        L.covgpu_aggregate.argtypes = [vp, C.c_int, C.c_int, i32p, f64p, vp, f64p, f64p]
        L.covgpu_learned_features.argtypes = [vp, C.POINTER(Params), C.c_double, C.c_int, C.c_int, f32p]
        L.covgpu_rscape_learned.argtypes = [vp, C.POINTER(Params), vp, vp, vp, C.c_double, C.c_int, C.c_int,
                                            C.POINTER(Result), C.POINTER(Hit), C.c_int, C.POINTER(C.c_int)]
        L.covgpu_pair_classes.argtypes = [vp, C.c_int, vp, vp, vp]
        L.covgpu_batch_create.argtypes = [C.POINTER(vp), C.c_int, C.c_double]
        L.covgpu_batch_destroy.argtypes = [vp]
        L.covgpu_batch_errmsg.argtypes = [vp]
        L.covgpu_batch_errmsg.restype = C.c_char_p
        L.covgpu_rscape_families.argtypes = [vp, C.POINTER(Params), C.c_int, C.POINTER(Family), C.c_int, i32p,
                                             C.POINTER(Result), C.POINTER(Hit), C.c_int]
        L.covgpu_batch_timing.argtypes = [vp, f64p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.covgpu_batch_set_schedule.argtypes = [vp, C.c_int, C.c_int]
        L.covgpu_batch_autotune.argtypes = [vp, C.POINTER(Params), C.c_int, C.POINTER(Family), C.c_int, i32p, C.c_int,
                                            i32p, C.c_int, i32p, f64p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        _LIB = L
    return _LIB


def default_allow():
    a = np.zeros(16)
    for x, y in ((0, 3), (3, 0), (1, 2), (2, 1), (2, 3), (3, 2)):
        a[x * 4 + y] = 1.0
    return a


SAMPLE_CONTACTS, SAMPLE_BP, SAMPLE_WC, SAMPLE_ALL = 0, 1, 2, 3


def params(**kw):
    """covgpu_params with the defaults of covgpu_params_default, overridden
    by kw.  contacts = [(i, j, bptype), ...] (1-based columns, i < j) gives
    the structure of the two-set test (with samplesize); the arrays are kept
    alive on the returned object."""
    p = Params()
    lib().covgpu_params_default(C.byref(p))
    keep = []
    for k, v in kw.items():
        if k == "allow":
            for i in range(16):
                p.allow[i] = float(v[i])
            continue
        if k == "contacts":
            c = np.asarray(v, dtype=np.int64).reshape(-1, 3)
            ci, cj = np.ascontiguousarray(c[:, 0]), np.ascontiguousarray(c[:, 1])
            ct = np.ascontiguousarray(c[:, 2].astype(np.int32))
            keep += [ci, cj, ct]
            p.ncnt, p.cnt_i, p.cnt_j, p.cnt_type = len(c), ci.ctypes.data, cj.ctypes.data, ct.ctypes.data
            continue
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    p._keep = keep
    return p


class Synth:
    """A synthetic alignment with its generating tree and planted structure."""

    def __init__(self, N, L, tree_len, nbp, nhelix, hmin, hmax, gap_rate, gap_mean=3.0, seed=42, tree_kind=0):
        self.ax = np.zeros((N, L), dtype=np.uint8)
        self.parent = np.zeros(N - 1, dtype=np.int32)
        self.left = np.zeros(N - 1, dtype=np.int32)
        self.right = np.zeros(N - 1, dtype=np.int32)
        self.ld = np.zeros(N - 1)
        self.rd = np.zeros(N - 1)
        self.ct = np.zeros(L, dtype=np.int32)
        st = lib().covgpu_synth2(N, L, tree_kind, tree_len, nbp, nhelix, hmin, hmax, gap_rate, gap_mean, seed,
                                 self.ax, self.parent, self.left, self.right, self.ld, self.rd, self.ct)
        if st:
            raise ValueError("covgpu_synth: bad sizes (status %d)" % st)


def synth_model():
    """(Q4, pi4, Q16, pi16) of the synthetic-alignment model."""
    Q4, pi4, Q16, pi16 = np.zeros(16), np.zeros(4), np.zeros(256), np.zeros(16)
    lib().covgpu_synth_model(Q4, pi4, Q16, pi16)
    return Q4.reshape(4, 4), pi4, Q16.reshape(16, 16), pi16


def weights_pb(ax):
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    w = np.zeros(ax.shape[0])
    lib().covgpu_weights_pb(ax, ax.shape[0], ax.shape[1], w)
    return w


def gapfilter(ax, wgt=None, gapthresh=0.75):
    ax = np.ascontiguousarray(ax, dtype=np.uint8)
    N, L = ax.shape
    w = np.ones(N) if wgt is None else np.ascontiguousarray(wgt, dtype=np.float64)
    use = np.zeros(L, dtype=np.int32)
    lib().covgpu_gapfilter(ax, w, N, L, gapthresh, use)
    return use.astype(bool)


# Easel's digital RNA alphabet: codes 0-3 the residues, 4 the gap, 5-15 the
# degeneracies, 16 the nonresidue, 17 the missing-data symbol
RNA_SYMBOLS = "ACGU-RYMKSWHBVDN*~"


def write_stockholm(path, ax, names=None, msa_name=None, append=False):
    """An alignment of Easel digital RNA codes [N][L] as one Stockholm record
    (header, #=GF ID when msa_name is given, one line per sequence, //): the
    format R-scape's --outnull writes its null alignments in
    (src/R-scape.c:1645-1672, one esl_msafile_Write record per null).  With
    append=True the records of several alignments go to one file."""
    ax = np.asarray(ax, dtype=np.uint8)
    if ax.ndim != 2 or (ax.size and int(ax.max()) >= len(RNA_SYMBOLS)):
        raise ValueError("codes must be a 2-D array of values below %d" % len(RNA_SYMBOLS))
    N = ax.shape[0]
    names = ["seq%d" % (k + 1) for k in range(N)] if names is None else [str(n) for n in names]
    if len(names) != N or any((not n) or any(ch.isspace() for ch in n) for n in names):
        raise ValueError("one non-empty name without spaces per sequence")
    table = np.frombuffer(RNA_SYMBOLS.encode(), dtype=np.uint8)
    width = max(len(n) for n in names) if N else 0
    with open(path, "a" if append else "w") as fh:
        fh.write("# STOCKHOLM 1.0\n")
        if msa_name:
            fh.write("#=GF ID %s\n" % msa_name)
        fh.write("\n")
        for n, row in zip(names, ax):
            fh.write("%-*s %s\n" % (width, n, table[row].tobytes().decode()))
        fh.write("//\n")


def read_stockholm(path):
    """The records of a Stockholm file as (ID or None, names, codes [N][L])
    tuples, for records written one line per sequence (write_stockholm's
    form); the residues are mapped to Easel digital RNA codes (T as U, '.'
    as a gap, lower case as upper case)."""
    look = {ch: k for k, ch in enumerate(RNA_SYMBOLS)}
    look.update({"T": 3, ".": 4, "_": 4})
    out, name, names, rows = [], None, [], []
    for line in open(path):
        line = line.rstrip("\n")
        if line.startswith("//"):
            ax = np.array([[look[ch] for ch in r.upper()] for r in rows], dtype=np.uint8)
            out.append((name, names, ax.reshape(len(rows), -1)))
            name, names, rows = None, [], []
        elif line.startswith("#=GF ID"):
            name = line.split(None, 2)[2].strip()
        elif line.strip() and not line.startswith("#"):
            n, r = line.split()
            names.append(n)
            rows.append(r)
    return out


AGG_FISHER, AGG_LANCASTER, AGG_WFISHER, AGG_SIDAK = 0, 1, 2, 3


def helices(ct, helix_unpaired=2):
    """R-scape's helices of a nested structure ct (0-based partner or -1):
    list of [(i, j), ...] per helix, each in increasing i."""
    ct = np.ascontiguousarray(ct, dtype=np.int32)
    L = len(ct)
    off = np.zeros(L // 2 + 2, dtype=np.int32)
    bi = np.zeros(L // 2 + 1, dtype=np.int32)
    bj = np.zeros(L // 2 + 1, dtype=np.int32)
    nh = C.c_int(0)
    st = lib().covgpu_helices(ct, L, helix_unpaired, C.byref(nh), off, bi, bj)
    if st:
        raise ValueError("covgpu_helices: status %d" % st)
    return [[(int(bi[k]), int(bj[k])) for k in range(off[h], off[h + 1])] for h in range(nh.value)]


class Engine:
    """One device context for alignments of N x L."""

    def __init__(self, N, L, maxslots=1, maxnull=0, device=0):
        self.N, self.L = N, L
        self.h = C.c_void_p()
        st = lib().covgpu_create(C.byref(self.h), device, N, L, maxslots, maxnull)
        if st:
            msg = lib().covgpu_errmsg(self.h).decode() if self.h else ""
            self.close()
            raise RuntimeError("covgpu_create failed (%d): %s" % (st, msg))

    def resize(self, N, L):
        """Work on alignments of N x L (within the dimensions the context was made for)."""
        self._ck(lib().covgpu_resize(self.h, N, L))
        self.N, self.L = N, L

    def close(self):
        if self.h:
            lib().covgpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st):
        if st:
            raise RuntimeError("covgpu error %d: %s" % (st, lib().covgpu_errmsg(self.h).decode()))

    def set_weights(self, wgt):
        self._ck(lib().covgpu_set_weights(self.h, np.ascontiguousarray(wgt, dtype=np.float64)))

    def set_alignment(self, slot, ax):
        self._ck(lib().covgpu_set_alignment(self.h, slot, np.ascontiguousarray(ax, dtype=np.uint8)))

    def get_alignment(self, slot):
        out = np.zeros((self.N, self.L), dtype=np.uint8)
        self._ck(lib().covgpu_get_alignment(self.h, slot, out))
        return out

    def write_nulls(self, path, first_slot, nslots, names=None, msa_name="null"):
        """The alignments in slots first_slot .. first_slot+nslots-1 (the null
        alignments after make_nulls, or after rscape) into one Stockholm file,
        one record per alignment named msa_name + index, as R-scape's --outnull
        writes its nulls (src/R-scape.c:1645-1672)."""
        open(path, "w").close()
        for k in range(nslots):
            write_stockholm(path, self.get_alignment(first_slot + k), names, "%s%d" % (msa_name, k + 1),
                            append=True)

    def set_tree(self, parent, left, right):
        self._ck(lib().covgpu_set_tree(self.h, np.ascontiguousarray(parent, dtype=np.int32),
                                       np.ascontiguousarray(left, dtype=np.int32),
                                       np.ascontiguousarray(right, dtype=np.int32)))

    def make_nulls(self, seed, first_null, nnull, first_slot):
        self._ck(lib().covgpu_make_nulls(self.h, seed, first_null, nnull, first_slot))

    def simulate(self, ld, rd, Q4, pi4, Q16, pi16, ct, root=None, gap_rate=0.0, gap_mean=0.0, seed=42, rep0=0,
                 first_slot=0, nrep=1):
        """nrep alignments evolved down the tree set by set_tree (branch lengths ld, rd)
        into slots first_slot..; see covgpu_simulate."""
        f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        rt = None if root is None else np.ascontiguousarray(root, dtype=np.uint8)
        self._ck(lib().covgpu_simulate(self.h, f(ld), f(rd), f(Q4), f(pi4), f(Q16), f(pi16),
                                       np.ascontiguousarray(ct, dtype=np.int32),
                                       None if rt is None else rt.ctypes.data, float(gap_rate), float(gap_mean),
                                       seed, rep0, first_slot, nrep))

    def weights_pb(self, slot=0, set=True):
        """Position-based weights of the alignment in slot, computed on the device."""
        w = np.zeros(self.N)
        self._ck(lib().covgpu_weights_pb_dev(self.h, slot, 1 if set else 0, w))
        return w

    def substitutions(self, slot=0, seed=42, includegaps=False):
        """(nsubs[L], ndouble[L,L], njoin[L,L]) on the Fitch reconstruction of the alignment in slot."""
        ns = np.zeros(self.L, dtype=np.int32)
        nd = np.zeros((self.L, self.L), dtype=np.int32)
        nj = np.zeros((self.L, self.L), dtype=np.int32)
        self._ck(lib().covgpu_substitutions(self.h, slot, seed, 1 if includegaps else 0, ns, nd, nj))
        return ns, nd, nj

    def power(self, single=None, join=None, double=None):
        """Pair power (i < j, row-major) from step curves given as (subs, prob) arrays of one length."""
        curves = [single, join, double]
        ns = max([len(c[0]) for c in curves if c is not None] + [0])
        keep = []
        def ptr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return a.ctypes.data
        args = []
        for c in curves:
            args += [ptr(None if c is None else c[0]), ptr(None if c is None else c[1])]
        P = self.L * (self.L - 1) // 2
        outs = [np.zeros(P) for _ in range(3)]
        self._ck(lib().covgpu_power(self.h, ns, *args, *[o.ctypes.data for o in outs]))
        return outs

    def pair_classes(self, slot=0):
        """(Watson-Crick, wobble, non-canonical) pair fractions of power_SPAIR_AddMI for
        every pair i < j (row-major), from the last scoring's counts of slot."""
        P = self.L * (self.L - 1) // 2
        out = [np.zeros(P) for _ in range(3)]
        self._ck(lib().covgpu_pair_classes(self.h, slot, *[o.ctypes.data for o in out]))
        return out

    def weights_gsc(self, slot=0, set=True):
        """GSC tree weights of the alignment in slot, computed on the device."""
        w = np.zeros(self.N)
        self._ck(lib().covgpu_weights_gsc_dev(self.h, slot, 1 if set else 0, w))
        return w

    def gapfilter(self, slot=0, wgt=None, gapthresh=0.75):
        """Columns of the alignment in slot that the gap filter keeps (bool[L])."""
        use = np.zeros(self.L, dtype=np.int32)
        wv = None if wgt is None else np.ascontiguousarray(wgt, dtype=np.float64)
        self._ck(lib().covgpu_gapfilter_dev(self.h, slot, None if wv is None else wv.ctypes.data, gapthresh, use))
        return use.astype(bool)

    def sim_tables(self):
        nb = 2 * (self.N - 1)
        P4 = np.zeros(nb * 16)
        P16 = np.zeros(nb * 256)
        self._ck(lib().covgpu_sim_tables(self.h, P4, P16))
        return P4.reshape(nb, 4, 4), P16.reshape(nb, 16, 16)

    def score(self, types, first_slot=0, nslots=1, covclass=CSELECT, nseqthresh=8, alenthresh=50, allow=None,
              counter=SIMT):
        codes = np.array([covtype_code(t) for t in types], dtype=np.int32)
        allow = default_allow() if allow is None else np.ascontiguousarray(allow, dtype=np.float64)
        mm = np.zeros(nslots * len(codes) * 2)
        self._ck(lib().covgpu_score(self.h, first_slot, nslots, len(codes), codes, covclass, nseqthresh, alenthresh,
                                    allow, counter, mm))
        return mm.reshape(nslots, len(codes), 2)

    def get_cov(self, slot, which=0):
        out = np.zeros(self.L * self.L)
        self._ck(lib().covgpu_get_cov(self.h, slot, which, out))
        return out.reshape(self.L, self.L)

    def get_probs(self, slot, wgt=None):
        L = self.L
        pp = np.zeros(L * L * 16)
        ne = np.zeros(L * L)
        ng = np.zeros(L * L)
        pm = np.zeros(L * 4)
        ps = np.zeros(L * 5)
        wp = None if wgt is None else np.ascontiguousarray(wgt, dtype=np.float64)
        self._ck(lib().covgpu_get_probs(self.h, slot, wp.ctypes.data if wp is not None else None, pp.ctypes.data,
                                        ne.ctypes.data, ng.ctypes.data, pm.ctypes.data, ps.ctypes.data))
        return pp.reshape(L, L, 16), ne.reshape(L, L), ng.reshape(L, L), pm.reshape(L, 4), ps.reshape(L, 5)

    def rscape(self, ax, wgt, types, hitcap=1 << 16, **kw):
        """ax / wgt = None reuse what is already on the device."""
        p = params(**kw)
        codes = np.array([covtype_code(t) for t in types], dtype=np.int32)
        res = (Result * len(codes))()
        hits = (Hit * (len(codes) * hitcap))()
        axc = None if ax is None else np.ascontiguousarray(ax, dtype=np.uint8)
        wc = None if wgt is None else np.ascontiguousarray(wgt, dtype=np.float64)
        self._ck(lib().covgpu_rscape(self.h, C.byref(p), axc.ctypes.data if axc is not None else None,
                                     wc.ctypes.data if wc is not None else None, len(codes), codes, res, hits,
                                     hitcap))
        out = []
        for q in range(len(codes)):
            r = {f[0]: getattr(res[q], f[0]) for f in Result._fields_}
            n = min(r["nhit"], hitcap)
            r["hits"] = [(hits[q * hitcap + k].i, hits[q * hitcap + k].j, hits[q * hitcap + k].sc,
                          hits[q * hitcap + k].E, hits[q * hitcap + k].pval) for k in range(n)]
            out.append(r)
        return out

    def features(self, slot=0, tree_len=0.0):
        """Features 0-46 of the learned null for the alignment in slot (float32[64], 47-63 zero)."""
        f = np.zeros(64, dtype=np.float32)
        self._ck(lib().covgpu_features(self.h, slot, float(tree_len), f))
        return f

    def learned_features(self, tree_len, nquick=4, covtype="GTp", **kw):
        """All 64 learned-null features of slot 0 (with nquick simulated nulls)."""
        p = params(**kw)
        f = np.zeros(64, dtype=np.float32)
        self._ck(lib().covgpu_learned_features(self.h, C.byref(p), float(tree_len), covtype_code(covtype), nquick, f))
        return f

    def rscape_learned(self, ax, wgt, net, tree_len, covtype="GTp", nquick=4, hitcap=1 << 16, **kw):
        """covgpu_rscape with the learned null; returns (result dict, used_net)."""
        p = params(**kw)
        res = Result()
        hits = (Hit * hitcap)()
        used = C.c_int(0)
        axc = None if ax is None else np.ascontiguousarray(ax, dtype=np.uint8)
        wc = None if wgt is None else np.ascontiguousarray(wgt, dtype=np.float64)
        self._ck(lib().covgpu_rscape_learned(self.h, C.byref(p), axc.ctypes.data if axc is not None else None,
                                             wc.ctypes.data if wc is not None else None, net.h, float(tree_len),
                                             covtype_code(covtype), nquick, C.byref(res), hits, hitcap,
                                             C.byref(used)))
        r = {f[0]: getattr(res, f[0]) for f in Result._fields_}
        n = min(r["nhit"], hitcap)
        r["hits"] = [(hits[k].i, hits[k].j, hits[k].sc, hits[k].E, hits[k].pval) for k in range(n)]
        return r, bool(used.value)

    def aggregate(self, method, helix_pvals, aux=None):
        """Aggregated p-values and E-values of helices given as lists of pair p-values."""
        off = np.zeros(len(helix_pvals) + 1, dtype=np.int32)
        off[1:] = np.cumsum([len(h) for h in helix_pvals])
        pv = np.ascontiguousarray(np.concatenate([np.asarray(h, float) for h in helix_pvals])
                                  if helix_pvals else np.zeros(0), dtype=np.float64)
        ax = None if aux is None else np.ascontiguousarray(np.concatenate([np.asarray(a, float) for a in aux]))
        pagg = np.zeros(len(helix_pvals))
        Eagg = np.zeros(len(helix_pvals))
        self._ck(lib().covgpu_aggregate(self.h, method, len(helix_pvals), off, pv,
                                        ax.ctypes.data if ax is not None else None, pagg, Eagg))
        return pagg, Eagg

    def autotune(self, nslots, first_slot=0, candidates=(4, 6, 8, 10, 12, 16, 24, 32004, 48004, 48008, 96004)):
        """Pick the tensor count kernel's raster super-block on these alignments: (best, {size: ms}).
        A size below 1000 is a square super-block; 1000 a + b is a band a tile rows high, b wide."""
        cand = np.ascontiguousarray(candidates, dtype=np.int32)
        ms = np.zeros(len(cand), dtype=np.float32)
        best = C.c_int(0)
        self._ck(lib().covgpu_autotune(self.h, first_slot, nslots, len(cand), cand.ctypes.data, ms, C.byref(best)))
        return best.value, {int(c): float(m) for c, m in zip(cand, ms)}

    def flush_l2(self):
        self._ck(lib().covgpu_flush_l2(self.h))

    def last_timing(self):
        ms = np.zeros(5)
        n = C.c_int()
        lib().covgpu_last_timing(self.h, ms, C.byref(n))
        return ms, n.value


NPARAM = 148995


class MLP:
    """The learned-null network on one device (include/covgpu.h, covgpu_mlp_*)."""

    def __init__(self, batch_cap=512, seed=1, device=0):
        self.h = C.c_void_p()
        st = lib().covgpu_mlp_create(C.byref(self.h), device, batch_cap, seed)
        if st:
            msg = lib().covgpu_mlp_errmsg(self.h) if self.h else b""
            lib().covgpu_mlp_destroy(self.h)
            self.h = None
            raise RuntimeError("covgpu_mlp_create failed (%d): %s" % (st, msg.decode() if msg else ""))

    def close(self):
        if self.h:
            lib().covgpu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st):
        if st:
            raise RuntimeError("covgpu_mlp error %d: %s" % (st, lib().covgpu_mlp_errmsg(self.h).decode()))

    def params(self):
        p = np.zeros(NPARAM, dtype=np.float32)
        self._ck(lib().covgpu_mlp_get_params(self.h, p))
        return p

    def set_params(self, p):
        self._ck(lib().covgpu_mlp_set_params(self.h, np.ascontiguousarray(p, dtype=np.float32)))

    def set_members(self, params):
        """An ensemble: params[k] (k < 16) are the members' parameters; forward
        averages their standardised outputs.  An empty list restores the
        single network."""
        P = np.ascontiguousarray(np.asarray(params, dtype=np.float32).reshape(-1, NPARAM))
        self._ck(lib().covgpu_mlp_set_members(self.h, P.ctypes.data if len(P) else None, len(P)))

    def set_norm(self, xmean, xstd, ymean, ystd, xlo=None, xhi=None):
        f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32)
        lo, hi = f(xlo), f(xhi)
        self._keep = (lo, hi)
        self._ck(lib().covgpu_mlp_set_norm(self.h, f(xmean), f(xstd), f(ymean), f(ystd),
                                           lo.ctypes.data if lo is not None else None,
                                           hi.ctypes.data if hi is not None else None))

    def norm(self):
        out = [np.zeros(64, np.float32), np.zeros(64, np.float32), np.zeros(3, np.float32), np.zeros(3, np.float32),
               np.zeros(64, np.float32), np.zeros(64, np.float32)]
        self._ck(lib().covgpu_mlp_get_norm(self.h, *out))
        return out

    def norm_vector(self):
        xm, xs, ym, ys, _, _ = self.norm()
        return np.concatenate([xm, xs, ym, ys]).astype(np.float32)

    def in_range(self, feat):
        return bool(lib().covgpu_mlp_in_range(self.h, np.ascontiguousarray(feat, dtype=np.float32)))

    def forward(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, 64)
        Y = np.zeros((X.shape[0], 3), dtype=np.float32)
        self._ck(lib().covgpu_mlp_forward(self.h, X, X.shape[0], Y))
        return Y

    def grad(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, 64)
        T = np.ascontiguousarray(T, dtype=np.float32).reshape(-1, 3)
        g = np.zeros(NPARAM, dtype=np.float32)
        loss = C.c_float(0)
        self._ck(lib().covgpu_mlp_grad(self.h, X, T, X.shape[0], g, C.byref(loss)))
        return loss.value, g

    def train(self, X, T, epochs, batch=256, lr=1e-3, wd=1e-4, seed=1):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, 64)
        T = np.ascontiguousarray(T, dtype=np.float32).reshape(-1, 3)
        hist = np.zeros(epochs, dtype=np.float32)
        self._ck(lib().covgpu_mlp_train(self.h, X, T, X.shape[0], epochs, batch, lr, wd, seed, hist))
        return hist


class Batch:
    """The E-valued path over a batch of alignment families on one device
    (include/covgpu.h, covgpu_rscape_families)."""

    def __init__(self, device=0, mem_gb=0.0):
        self.h = C.c_void_p()
        st = lib().covgpu_batch_create(C.byref(self.h), device, float(mem_gb))
        if st:
            msg = lib().covgpu_batch_errmsg(self.h).decode() if self.h else ""
            self.close()
            raise RuntimeError("covgpu_batch_create failed (%d): %s" % (st, msg))

    def close(self):
        if self.h:
            lib().covgpu_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _families(families):
        keep = []
        fam = (Family * max(len(families), 1))()
        for k, f in enumerate(families):
            ax = np.ascontiguousarray(f["ax"], dtype=np.uint8)
            keep.append(ax)
            fam[k].N, fam[k].L = ax.shape
            fam[k].ax = ax.ctypes.data
            for name in ("wgt", "parent", "left", "right"):
                v = f.get(name)
                if v is None:
                    setattr(fam[k], name, None)
                    continue
                a = np.ascontiguousarray(v, dtype=np.float64 if name == "wgt" else np.int32)
                keep.append(a)
                setattr(fam[k], name, a.ctypes.data)
        return fam, keep

    def set_schedule(self, simt_below, sb):
        """Families of fewer than simt_below sequences count on the SIMT kernel; sb the raster super-block."""
        if lib().covgpu_batch_set_schedule(self.h, int(simt_below), int(sb)):
            raise ValueError("bad schedule")

    def autotune(self, families, types, thr=(0, 64, 128, 256), sb=(6, 10, 16), **kw):
        """Time the families under every (threshold, super-block) pair and keep the
        fastest: (best threshold, best super-block, {(thr, sb): seconds})."""
        p = params(**kw)
        codes = np.array([covtype_code(t) for t in types], dtype=np.int32)
        fam, keep = self._families(families)
        th = np.ascontiguousarray(thr, dtype=np.int32)
        sbs = np.ascontiguousarray(sb, dtype=np.int32)
        ms = np.zeros(len(th) * len(sbs))
        bt, bs = C.c_int(), C.c_int()
        st = lib().covgpu_batch_autotune(self.h, C.byref(p), len(families), fam, len(codes), codes, len(th), th,
                                         len(sbs), sbs, ms, C.byref(bt), C.byref(bs))
        if st:
            raise RuntimeError("covgpu batch error %d: %s" % (st, lib().covgpu_batch_errmsg(self.h).decode()))
        times = {(int(a), int(c)): float(ms[i * len(sbs) + j]) / 1000.0 for i, a in enumerate(th)
                 for j, c in enumerate(sbs)}
        return bt.value, bs.value, times

    def rscape(self, families, types, hitcap=1 << 12, **kw):
        """families: dicts with ax [N][L] (uint8), parent/left/right (int32,
        N-1 each; parent optional) and optionally wgt [N] (None: R-scape's rule
        on the device).  Returns, per family, the list of result dicts of
        covgpu_rscape (one per type)."""
        p = params(**kw)
        codes = np.array([covtype_code(t) for t in types], dtype=np.int32)
        nf, nt = len(families), len(codes)
        fam, keep = self._families(families)
        res = (Result * max(nf * nt, 1))()
        hits = (Hit * max(nf * nt * hitcap, 1))()
        st = lib().covgpu_rscape_families(self.h, C.byref(p), nf, fam, nt, codes, res, hits, hitcap)
        if st:
            raise RuntimeError("covgpu batch error %d: %s" % (st, lib().covgpu_batch_errmsg(self.h).decode()))
        out = []
        for k in range(nf):
            rows = []
            for q in range(nt):
                e = k * nt + q
                r = {f[0]: getattr(res[e], f[0]) for f in Result._fields_}
                n = min(r["nhit"], hitcap)
                b = e * hitcap
                r["hits"] = [(hits[b + i].i, hits[b + i].j, hits[b + i].sc, hits[b + i].E, hits[b + i].pval)
                             for i in range(n)]
                rows.append(r)
            out.append(rows)
        return out

    def timing(self):
        """(ms of the passes to the corrected scores, ms of the rest, host ms
        of the call, kernel launches, chunks) of the last call."""
        ms = np.zeros(3)
        n, c = C.c_int(), C.c_int()
        lib().covgpu_batch_timing(self.h, ms, C.byref(n), C.byref(c))
        return ms[0], ms[1], ms[2], n.value, c.value
