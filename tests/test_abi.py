"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares (no compute calls here)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(path):
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set()
    for m in re.finditer(r"^\s*(?:extern\s+)?[A-Za-z_][\w\s\*]*?\b([a-z][A-Za-z0-9_]+)\s*\(", src, flags=re.M):
        name = m.group(1)
        if name in ("if", "for", "while", "return", "sizeof"):
            continue
        names.add(name)
    return names


def test_headers_parse():
    names = declared(os.path.join(ROOT, "include", "rscape_cov.h"))
    assert "corr_CalculateGT" in names and "cov_Calculate" in names
    names = declared(os.path.join(ROOT, "include", "covgpu.h"))
    assert "covgpu_rscape" in names


@pytest.mark.parametrize("header", ["covgpu.h", "rscape_cov.h"])
def test_every_declared_symbol_is_exported(covgpu, header):
    lib = ctypes.CDLL(covgpu.LIBPATH)
    missing = [n for n in sorted(declared(os.path.join(ROOT, "include", header))) if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_entry_points_present(covgpu):
    """The correlators.h / covariation.h names the hot path binds."""
    lib = ctypes.CDLL(covgpu.LIBPATH)
    for n in ["corr_Create", "corr_Reuse", "corr_ReuseCOV", "corr_Destroy", "corr_NaivePP", "corr_NaivePS",
              "corr_Marginals", "corr_Probs", "corr_ValidateProbs", "corr_CalculateCHI", "corr_CalculateCHI_C16",
              "corr_CalculateCHI_C2", "corr_CalculateOMES", "corr_CalculateOMES_C16", "corr_CalculateOMES_C2",
              "corr_CalculateGT", "corr_CalculateGT_C16", "corr_CalculateGT_C2", "corr_CalculateGT_CWC",
              "corr_CalculateMI", "corr_CalculateMI_C16", "corr_CalculateMI_C2", "corr_CalculateMIr",
              "corr_CalculateMIr_C16", "corr_CalculateMIr_C2", "corr_CalculateMIg", "corr_CalculateMIg_C16",
              "corr_CalculateMIg_C2", "corr_CalculateRAF", "corr_CalculateRAFS", "corr_CalculateCCF",
              "corr_CalculateCCF_C16", "corr_CalculateCOVCorrected", "corr_COVTYPEString", "corr_String2COVTYPE",
              "cov_Calculate", "cov_SignificantPairs_Ranking", "cov_CreateRankList", "cov_GrowRankList",
              "cov_CreateHitList", "cov_NullFitGamma", "cov_NullFitExponential", "cov_histogram_SetSurvFitTail",
              "cov_ReadNullHistogram", "cov_WriteNullHistogram", "cov_ranklist_Bin2Bin", "cov_FreeRankList",
              "cov_FreeHitList"]:
        assert hasattr(lib, n), n


def test_host_utilities_without_gpu(covgpu):
    """Synthetic alignments, weights and the gap filter are host code."""
    import numpy as np
    s = covgpu.Synth(50, 80, 1.5, 12, 2, 6, 6, 0.1, seed=3)
    assert s.ax.shape == (50, 80) and s.ax.max() <= 4
    # Easel convention: parent < child for internal nodes, every leaf once
    leaves = sorted([-c for c in np.concatenate([s.left, s.right]) if c <= 0])
    assert leaves == list(range(50))
    for v in range(49):
        for c in (s.left[v], s.right[v]):
            if c > 0:
                assert c > v and s.parent[c] == v
    assert np.sum(s.ct >= 0) == 24
    for i in np.nonzero(s.ct >= 0)[0]:
        assert s.ct[s.ct[i]] == i
    gap = np.mean(s.ax == 4)
    assert 0.04 < gap < 0.2
    w = covgpu.weights_pb(s.ax)
    assert abs(w.sum() - 50) < 1e-9
    assert covgpu.gapfilter(s.ax).all()


def test_host_weights_match_oracle(covgpu, oracle):
    s = covgpu.Synth(40, 60, 1.0, 0, 0, 0, 0, 0.1, seed=9)
    import numpy as np
    assert np.allclose(covgpu.weights_pb(s.ax), oracle.weights_pb(s.ax), rtol=1e-12)
    assert np.array_equal(covgpu.gapfilter(s.ax, None, 0.5), oracle.gapfilter(s.ax, None, 0.5))


def test_histogram_io_roundtrip(covgpu, tmp_path):
    """cov_WriteNullHistogram / cov_ReadNullHistogram keep 'score count'
    lines (src/covariation.c:1717-1867)."""
    lib = ctypes.CDLL(covgpu.LIBPATH)
    lib.cov_CreateRankList.restype = ctypes.c_void_p
    lib.cov_CreateRankList.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double]
    lib.cov_WriteNullHistogram.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
    lib.cov_ReadNullHistogram.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p,
                                          ctypes.c_int]
    lib.cov_FreeRankList.argtypes = [ctypes.c_void_p]
    lib.covh_Add.argtypes = [ctypes.c_void_p, ctypes.c_double]
    r = lib.cov_CreateRankList(20.0, -10.0, 0.5)
    ha = ctypes.cast(r, ctypes.POINTER(ctypes.c_void_p))[0]
    for x in (-3.2, 0.1, 0.2, 4.9, 4.9, 17.0):
        assert lib.covh_Add(ha, x) == 0
    f = str(tmp_path / "null.his").encode()
    eb = ctypes.create_string_buffer(256)
    assert lib.cov_WriteNullHistogram(f, r, eb, 0) == 0
    r2 = ctypes.c_void_p()
    assert lib.cov_ReadNullHistogram(f, ctypes.byref(r2), eb, 0) == 0
    lines = [l.split() for l in open(f.decode())]
    assert sum(int(c) for s, c in lines) == 6
    lib.cov_FreeRankList(r)
    lib.cov_FreeRankList(r2)


def test_null_merge_bin_mapping_matches_the_library(covgpu):
    """rscape_abi.bin2bin (the vectorised mapping of the callers' null
    merge, null_add2cumranklist at src/R-scape.c:1564-1612) gives the
    library's cov_ranklist_Bin2Bin for every bin, including halves and bins
    outside the target."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("rscape_abi", os.path.join(os.path.dirname(covgpu.LIBPATH),
                                                                               "rscape_abi.py"))
    abi = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(abi)
    lib = abi.setup_lib(covgpu.LIBPATH)
    rng = np.random.default_rng(3)
    cb = ctypes.c_int()
    for trial in range(60):
        w = float(rng.choice([0.05, 0.013, 0.0071, 1e-3, 0.25, 0.1]))
        bmin = float(rng.choice([-10.0, rng.uniform(-20, -5)]))
        rl = lib.cov_CreateRankList(float(rng.uniform(5, 60)), bmin, w)
        cum = lib.cov_CreateRankList(float(rng.uniform(5, 60)),
                                     float(rng.choice([bmin, bmin - 20 * w, rng.uniform(-30, bmin)])), w)
        h, c = rl.contents.ha.contents, cum.contents.ha.contents
        r, ok = abi.bin2bin(h, c, np.arange(h.nb))
        for k in range(h.nb):
            lib.cov_ranklist_Bin2Bin(k, rl.contents.ha, cum.contents.ha, ctypes.byref(cb))
            assert r[k] == (cb.value if 0 <= cb.value < c.nb else -1), (trial, k)
        lib.cov_FreeRankList(rl)
        lib.cov_FreeRankList(cum)


def test_default_parameters_are_the_reference_defaults(covgpu):
    """covgpu_params_default against R-scape's defaults: -E 0.05
    (src/R-scape.c:258), CSELECT with nseqthresh 8 and alenthresh 50 (:345-347),
    --tol 1e-6 (:426), --fracfit 1.0 and --pmass 0.0005 (:428-429), the null
    count chosen from the alignment size (:591), BMIN -10, HPTS 400 and W 0.05
    (src/covariation.h:22-24), and the allowed pairs A-U, C-G and G-U
    (src/R-scape.c:885-887), gamma tail fit."""
    p = covgpu.params()
    assert p.thresh == 0.05 and p.covclass == 3 and p.nseqthresh == 8 and p.alenthresh == 50
    assert p.tol == 1e-6 and p.fracfit == 1.0 and p.pmass == 0.0005 and p.nshuffle == -1
    assert p.bmin == -10.0 and p.hpts == 400 and p.w0 == 0.05 and p.doexpfit == 0
    allow = [p.allow[k] for k in range(16)]
    pairs = {(x, y) for x in range(4) for y in range(4) if allow[4 * x + y] > 0}
    assert pairs == {(0, 3), (3, 0), (1, 2), (2, 1), (2, 3), (3, 2)}


def test_histogram_bins_and_tail_survival(covgpu):
    """Easel's bin rule b = ceil((x - bmin)/w) - 1 puts a score on a bin's upper
    edge in that bin (bins are (lo, hi]), with the bounds bmin + b w and
    bmin + (b + 1) w; the gamma and exponential tail survival functions are
    Q(tau, lambda (x - mu)) and exp(-lambda (x - mu)) (scipy as the check)."""
    sp = pytest.importorskip("scipy.special")
    lib = ctypes.CDLL(covgpu.LIBPATH)
    lib.covh_Create.restype = ctypes.c_void_p
    lib.covh_Create.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double]
    lib.covh_Destroy.argtypes = [ctypes.c_void_p]
    lib.covh_Score2Bin.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
    lib.covh_Bin2LBound.restype = ctypes.c_double
    lib.covh_Bin2LBound.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.covh_Bin2UBound.restype = ctypes.c_double
    lib.covh_Bin2UBound.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.covh_gamma_surv.restype = ctypes.c_double
    lib.covh_gamma_surv.argtypes = [ctypes.c_double, ctypes.c_void_p]
    lib.covh_exp_surv.restype = ctypes.c_double
    lib.covh_exp_surv.argtypes = [ctypes.c_double, ctypes.c_void_p]
    h = lib.covh_Create(-10.0, 10.0, 0.5)
    b = ctypes.c_int()
    for k in range(1, 40):
        x = -10.0 + 0.5 * k                       # exactly on an edge
        assert lib.covh_Score2Bin(h, x, ctypes.byref(b)) == 0 and b.value == k - 1
        assert lib.covh_Score2Bin(h, x + 0.25, ctypes.byref(b)) == 0 and b.value == k
        assert lib.covh_Bin2LBound(h, k) == x and lib.covh_Bin2UBound(h, k) == x + 0.5
    lib.covh_Destroy(h)
    mu, lam, tau = 2.0, 0.7, 2.5
    gp = (ctypes.c_double * 3)(mu, lam, tau)
    ep = (ctypes.c_double * 2)(mu, lam)
    for x in (2.5, 4.0, 9.0, 30.0):
        assert lib.covh_gamma_surv(x, gp) == pytest.approx(sp.gammaincc(tau, lam * (x - mu)), rel=1e-10)
        assert lib.covh_exp_surv(x, ep) == pytest.approx(np.exp(-lam * (x - mu)), rel=1e-12)


def _abi(covgpu):
    import importlib.util
    spec = importlib.util.spec_from_file_location("rscape_abi", os.path.join(os.path.dirname(covgpu.LIBPATH),
                                                                               "rscape_abi.py"))
    abi = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(abi)
    return abi, abi.setup_lib(covgpu.LIBPATH)


def test_fisher_exact_test_is_the_hypergeometric_tail(covgpu):
    """cov_FisherExactTest (src/covariation.c:1584-1633): the probability of
    at least cNBP covarying pairs outside the BP base pairs, a hypergeometric
    upper tail over alen(alen-1)/2 + BP pairs."""
    from scipy.stats import hypergeom
    lib = ctypes.CDLL(covgpu.LIBPATH)
    lib.cov_FisherExactTest.argtypes = [ctypes.POINTER(ctypes.c_double)] + [ctypes.c_int] * 4
    for cBP, cNBP, BP, alen in ((3, 2, 20, 40), (10, 0, 30, 80), (0, 5, 12, 30), (7, 7, 25, 60)):
        p = ctypes.c_double()
        assert lib.cov_FisherExactTest(ctypes.byref(p), cBP, cNBP, BP, alen) == 0
        NBP = alen * (alen - 1) // 2
        ref = hypergeom.sf(cNBP - 1, BP + NBP, NBP, cBP + cNBP)
        assert p.value == pytest.approx(min(ref, 1.0), rel=1e-9, abs=1e-300)


def test_small_reference_entry_points(covgpu, tmp_path, capfd):
    """cov_THRESHTYPEString, cov_Add2SubsHistogram, cov_WriteHistogram's
    survival file (cov_histogram_PlotSurvival), cov_DumpRankList, and the
    refusals of corr_PostOrderPP and cov_CreateFOLDHitList."""
    abi, lib = _abi(covgpu)
    s = ctypes.c_char_p()
    lib.cov_THRESHTYPEString.argtypes = [ctypes.POINTER(ctypes.c_char_p), ctypes.c_int, ctypes.c_char_p]
    eb = ctypes.create_string_buffer(256)
    assert lib.cov_THRESHTYPEString(ctypes.byref(s), 0, eb) == 0 and s.value == b"Eval"
    assert lib.cov_THRESHTYPEString(ctypes.byref(s), 1, eb) != 0
    # WWc hits add nsubs + 1 to the substitution histogram
    hits = (abi.Hit * 4)()
    for k, (bpt, ns) in enumerate(((abi.WWc, 3), (abi.STACKED, 9), (abi.WWc, 0), (abi.BPNONE, 5))):
        hits[k].bptype, hits[k].nsubs = bpt, ns
    hl = abi.HitList(4, None, hits, 0, 0)
    rl = lib.cov_CreateRankList(20.0, 0.0, 1.0)
    h = rl.contents.ha
    lib.cov_Add2SubsHistogram.argtypes = [ctypes.POINTER(abi.Hist), ctypes.POINTER(abi.HitList), ctypes.c_int]
    assert lib.cov_Add2SubsHistogram(h, ctypes.byref(hl), 0) == 0
    hh = h.contents
    assert hh.Nc == 2 and hh.xmin == 1.0 and hh.xmax == 4.0
    # the survival file: ht's observed curve, hb's (empty), the null's
    lib.covh_Add.argtypes = [ctypes.POINTER(abi.Hist), ctypes.c_double]
    for x in (2.5, 3.5, 3.7, 8.0):
        lib.covh_Add(rl.contents.ht, x)
    data = abi.Data()
    data.errbuf = ctypes.cast(eb, ctypes.c_char_p)
    lib.cov_WriteHistogram.argtypes = [ctypes.POINTER(abi.Data), ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                       ctypes.c_int, ctypes.POINTER(abi.RankList), ctypes.c_char_p]
    f = tmp_path / "surv.txt"
    assert lib.cov_WriteHistogram(ctypes.byref(data), None, str(f).encode(), None, 3, rl, None) == 0
    lines = f.read_text().splitlines()
    assert lines[0] == "&"                                  # hb: empty
    body = lines[1:lines.index("&", 1)]
    # bins with data from the top: [8, 9) 1 of 4, [3, 4) 3 of 4, [2, 3) all
    assert [float(l.split("\t")[1]) for l in body] == [0.25, 0.75, 1.0]
    lib.cov_DumpRankList.argtypes = [ctypes.c_void_p, ctypes.POINTER(abi.RankList)]
    capfd.readouterr()
    assert lib.cov_DumpRankList(None, rl) == 0
    ctypes.CDLL(None).fflush(None)   # C's stdout buffer
    out = capfd.readouterr().out
    assert out.startswith("imin ") and "eval" in out
    lib.cov_FreeRankList(rl)
    lib.corr_PostOrderPP.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_double, ctypes.c_int, ctypes.c_char_p]
    assert lib.corr_PostOrderPP(None, None, None, None, 1e-6, 0, eb) != 0 and b"AKMAEV" in eb.value
    lib.cov_CreateFOLDHitList.argtypes = [ctypes.POINTER(abi.Data)] + [ctypes.c_void_p] * 8
    assert lib.cov_CreateFOLDHitList(ctypes.byref(data), None, None, None, None, None, None, None, None) != 0


def handle_entry_points(path):
    """(name, parameter count) of every function in a header whose first
    parameter is a context, batch or network handle."""
    src = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
    out = []
    for m in re.finditer(r"\bint\s+(covgpu_\w+)\s*\(\s*(?:const\s+)?covgpu_(?:ctx|batch|mlp)\s*\*\s*\w+([^;]*?)\)\s*;",
                         src, flags=re.S):
        rest = m.group(2).strip()
        out.append((m.group(1), 1 + (rest.count(",") if rest else 0)))
    return out


def test_null_handles_are_rejected(covgpu):
    """Every entry point that takes a context, batch or network returns 11
    for a NULL handle, before any device work (no GPU needed)."""
    lib = ctypes.CDLL(covgpu.LIBPATH)
    entries = handle_entry_points(os.path.join(ROOT, "include", "covgpu.h"))
    assert len(entries) > 40, entries
    for name, nargs in entries:
        f = getattr(lib, name)
        f.restype = ctypes.c_int
        got = f(*([None] * nargs))
        want = 0 if name == "covgpu_mlp_in_range" else 11   # a yes/no answer: not in range
        assert got == want, (name, got)


def test_stockholm_round_trip(covgpu, tmp_path):
    """Alignments written in R-scape's --outnull form (Stockholm, one record
    per alignment) read back code for code, every digital RNA code included."""
    rng = np.random.default_rng(4)
    a = rng.integers(0, 18, size=(7, 33)).astype(np.uint8)
    b = covgpu.Synth(12, 40, 1.0, 6, 1, 6, 6, 0.1, seed=9).ax
    path = str(tmp_path / "nulls.sto")
    covgpu.write_stockholm(path, a, msa_name="null1")
    covgpu.write_stockholm(path, b, names=["s%02d" % k for k in range(12)], msa_name="null2", append=True)
    text = open(path).read()
    assert text.startswith("# STOCKHOLM 1.0\n") and text.count("//\n") == 2
    recs = covgpu.read_stockholm(path)
    assert [r[0] for r in recs] == ["null1", "null2"]
    assert np.array_equal(recs[0][2], a) and np.array_equal(recs[1][2], b)
    assert recs[1][1][0] == "s00"
    with pytest.raises(ValueError):
        covgpu.write_stockholm(path, np.full((2, 3), 18, dtype=np.uint8))
    with pytest.raises(ValueError):
        covgpu.write_stockholm(path, a, names=["x y"] * 7)


@pytest.mark.parametrize("schedule", [1, 4, 10, 12, 24, 1001, 3005, 32004, 48008, 96004, 7001])
def test_count_schedules_cover_every_tile_once(covgpu, schedule):
    """Every raster the autotuner may pick (squares and bands) is a
    permutation of the upper-triangle tiles for the weighted count, and the
    unit-weight count's column-pair tasks cover each tile exactly once."""
    lib = ctypes.CDLL(covgpu.LIBPATH)
    for nT in list(range(1, 24)) + [47, 94, 188]:
        nt = nT * (nT + 1) // 2
        order = np.zeros(nt, dtype=np.int32)
        jp = np.zeros((nt, 4), dtype=np.int32)
        nj = ctypes.c_int()
        assert lib.covgpu_tile_order(nT, schedule, order.ctypes.data, jp.ctypes.data, nt, ctypes.byref(nj)) == 0
        assert np.array_equal(np.sort(order), np.arange(nt)), (nT, schedule)
        jp = jp[:nj.value]
        tiles = jp[:, 2:].ravel()
        tiles = tiles[tiles >= 0]
        assert np.array_equal(np.sort(tiles), np.arange(nt)), (nT, schedule)
        # the tiles of a task lie in its row I, at columns J0 and J0 + 1
        I, J0 = jp[:, 0], jp[:, 1]
        row0 = I * nT - I * (I - 1) // 2
        ok0 = jp[:, 2] < 0
        assert np.all(ok0 | (jp[:, 2] == row0 + J0 - I))
        ok1 = jp[:, 3] < 0
        assert np.all(ok1 | (jp[:, 3] == row0 + J0 + 1 - I))
        assert np.all(J0 % 2 == 0) and np.all(J0 + 1 >= I)


def test_count_schedule_rejects_bad_values(covgpu):
    lib = ctypes.CDLL(covgpu.LIBPATH)
    order = np.zeros(64, dtype=np.int32)
    nj = ctypes.c_int()
    for bad in (0, -3, 5000, 1000):
        assert lib.covgpu_tile_order(10, bad, order.ctypes.data, None, 0, ctypes.byref(nj)) == 11
    assert lib.covgpu_tile_order(0, 10, order.ctypes.data, None, 0, ctypes.byref(nj)) == 11


def test_headers_compile_as_c_and_link(covgpu, tmp_path):
    """include/covgpu.h and include/rscape_cov.h compile as strict C11 with
    every warning an error, and a C program links against libcovgpu and runs
    its host-only calls (no GPU)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "abi_check.c"
    src.write_text(r"""
#include <stdio.h>
#include "covgpu.h"
#include "rscape_cov.h"
int main(void) {
  covgpu_params p;
  int order[6], jp[24], nj = 0;
  covgpu_params_default(&p);
  if (p.nshuffle != -1 || p.thresh != 0.05) return 2;
  if (covgpu_tile_order(3, 10, order, jp, 6, &nj) != 0 || nj < 1) return 3;
  if (covgpu_rscape(NULL, &p, NULL, NULL, 1, NULL, NULL, NULL, 0) != 11) return 4;
  printf("ok %d\n", nj);
  return 0;
}
""")
    exe = tmp_path / "abi_check"
    libdir = os.path.dirname(covgpu.LIBPATH)
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src), "-o", str(exe), "-L", libdir, "-lcovgpu", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), (r.returncode, r.stdout, r.stderr)


def _c_layouts_match(tmp_path, incdir, header, pairs, cfield=None):
    """Compile a C program printing sizeof/offsetof of each C structure of
    pairs [(C type, ctypes class)] and compare with the ctypes layout."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    cfield = cfield or {}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "%s"' % header, "int main(void) {"]
    for cname, py in pairs:
        lines.append('  printf("%%s size %%zu\\n", "%s", sizeof(%s));' % (cname, cname))
        for f in py._fields_:
            lines.append('  printf("%%s %s %%zu\\n", "%s", offsetof(%s, %s));'
                         % (f[0], cname, cname, cfield.get((cname, f[0]), f[0])))
    lines += ["  return 0;", "}"]
    src = tmp_path / ("layout_%s.c" % header.replace(".", "_"))
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / ("layout_%s" % header.replace(".", "_"))
    r = subprocess.run([cc, "-std=c11", "-D_DEFAULT_SOURCE", "-I", incdir, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, timeout=60).stdout.splitlines():
        name, key, val = line.rsplit(" ", 2)
        got[(name, key)] = int(val)
    for cname, py in pairs:
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f in py._fields_:
            assert got[(cname, f[0])] == getattr(py, f[0]).offset, (cname, f[0])


def test_ctypes_mirrors_match_the_c_layouts(covgpu, tmp_path):
    """The ctypes structures of rscape_abi.py (the drop-in's Python binding,
    used by the tests and the benchmark) have the sizes and field offsets of
    the C structures in include/rscape_cov.h, as gcc lays them out."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("rscape_abi_t", os.path.join(ROOT, "r-scape_gb300", "rscape_abi.py"))
    abi = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(abi)
    pairs = [("ESL_ALPHABET", abi.Alphabet), ("ESL_MSA", abi.Msa), ("ESL_DMATRIX", abi.DMatrix),
             ("ESL_HISTOGRAM", abi.Hist), ("struct mutual_s", abi.Mutual), ("RANKLIST", abi.RankList),
             ("HIT", abi.Hit), ("HITLIST", abi.HitList), ("THRESH", abi.Thresh), ("ESL_RANDOMNESS", abi.Rand),
             ("CNT", abi.Cnt), ("CLIST", abi.Clist), ("struct data_s", abi.Data)]
    _c_layouts_match(tmp_path, os.path.join(ROOT, "include"), "rscape_cov.h", pairs,
                     {("struct data_s", "lambda_"): "lambda"})   # a Python keyword, renamed in the mirror


def test_covgpu_and_oracle_ctypes_mirrors_match(covgpu, oracle, tmp_path):
    """covgpu.py's mirrors of include/covgpu.h and oracle.py's mirrors of
    oracle/rscape_oracle.h have the C layouts."""
    _c_layouts_match(tmp_path, os.path.join(ROOT, "include"), "covgpu.h",
                     [("covgpu_params", covgpu.Params), ("covgpu_result", covgpu.Result), ("covgpu_hit", covgpu.Hit),
                      ("covgpu_family", covgpu.Family)],
                     {("covgpu_result", "lambda_"): "lambda"})
    _c_layouts_match(tmp_path, os.path.join(ROOT, "oracle"), "rscape_oracle.h",
                     [("orc_tree_t", oracle.Tree), ("orc_params_t", oracle.Params), ("orc_result_t", oracle.Result)],
                     {("orc_result_t", "lambda_"): "lambda"})
