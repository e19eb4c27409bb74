"""The deep-alignment workload at full size: N=20,000 x L=1,500 (tree length
2.5, 400 base pairs, 10% gaps, position-based weights), every statistic of
the tensor path (GT, CHI, MI, MIr, MIg, OMES, RAF, RAFS, CCF) raw and with
APC, against the FP64 oracle, each within 1e-5 relative (parity_tol).  The oracle forms the pair probabilities once (its
counting loop over the host threads) and every statistic and APC from
them; RAF and RAFS, whose reference loop is O(N^2) per pair, are checked on
sampled pairs.  The per-statistic maximum errors are printed and, with
COVGPU_ERROR_REPORT_DEEP set to a path, written there as JSON.
"""
import ctypes as C
import json
import os
import time

import numpy as np
import pytest

from parity_tol import stat_close

pytestmark = pytest.mark.gpu

N, L = 20000, 1500
STATS = {"CHI": 0, "GT": 3, "MI": 6, "MIr": 9, "MIg": 12, "OMES": 15}


def oracle_stat(oracle, code, pp, pm, nseff, ngap):
    COV = np.zeros(L * L)
    mm = np.zeros(2)
    st = oracle.lib().orc_stat(code, 3, N, L, 8, 50, pp.ravel(), pm.ravel(), nseff.ravel(), ngap.ravel(),
                               oracle.default_allow(), COV, mm)
    assert st == 0
    return COV


def oracle_apc(oracle, COV):
    out = COV.copy()
    mm = np.zeros(2)
    assert oracle.lib().orc_cov_corrected(0, L, out, mm) == 0
    return out


def test_deep_alignment_errors(covgpu, oracle):
    s = covgpu.Synth(N, L, 2.5, 400, 40, 6, 14, 0.10, seed=3)
    w = covgpu.weights_pb(s.ax)
    e = covgpu.Engine(N, L)
    e.set_weights(w)
    e.set_alignment(0, s.ax)
    iu = np.triu_indices(L, 1)
    got = {}
    t0 = time.perf_counter()
    for corr in ("", "p"):
        for group in (["GT", "CHI", "MI", "MIr"], ["OMES", "RAF", "RAFS", "CCF"], ["MIg"]):
            types = [t + corr for t in group]
            e.score(types, counter=covgpu.TENSOR)
            for q, t in enumerate(types):
                got[t] = e.get_cov(0, q)
    gpu_s = time.perf_counter() - t0
    e.close()
    # the oracle: probabilities once, every statistic and APC from them
    t0 = time.perf_counter()
    pp, nseff, ngap, pm, ps = oracle.probs(s.ax, w)
    ref = {}
    for t, code in STATS.items():
        ref[t] = oracle_stat(oracle, code, pp, pm, nseff, ngap)
    COV = np.zeros(L * L)
    mm = np.zeros(2)
    assert oracle.lib().orc_ccf(L, pm.ravel(), nseff.ravel(), COV, mm) == 0
    ref["CCF"] = COV
    for t in list(ref):
        ref[t + "p"] = oracle_apc(oracle, ref[t])
    oracle_s = time.perf_counter() - t0
    rows = []
    bad = []
    for t in ("CHI", "GT", "MI", "MIr", "MIg", "OMES", "CCF"):
        for name in (t, t + "p"):
            g = got[name].reshape(L, L)[iu]
            r = ref[name].reshape(L, L)[iu]
            ok, rel, small = stat_close(g, r)
            rows.append({"stat": name, "max_abs": float(np.abs(g - r).max()), "max_rel": rel,
                         "small_over_max": small})
            if not ok:
                bad.append(rows[-1])
    # RAF and RAFS on sampled pairs (RAFS needs the RAF of (i-1, j+1) and (i+1, j-1))
    rng = np.random.default_rng(7)
    pairs = set()
    while len(pairs) < 24:
        i = int(rng.integers(1, L - 4))
        j = int(rng.integers(i + 3, L - 1))
        pairs.add((i, j))
    pairs = sorted(pairs)
    need = sorted({q for (i, j) in pairs for q in ((i, j), (i - 1, j + 1), (i + 1, j - 1))})
    rafv = dict(zip(need, oracle.raf_pairs(s.ax, need)))
    graf = got["RAF"].reshape(L, L)
    grafs = got["RAFS"].reshape(L, L)
    erraf = max(abs(graf[i, j] - rafv[(i, j)]) for (i, j) in need)
    errafs = 0.0
    for (i, j) in pairs:
        v = 0.25 * (2 * rafv[(i, j)] + rafv[(i - 1, j + 1)] + rafv[(i + 1, j - 1)])
        errafs = max(errafs, abs(grafs[i, j] - v))
    rows.append({"stat": "RAF", "max_abs": float(erraf), "sampled_pairs": len(need)})
    rows.append({"stat": "RAFS", "max_abs": float(errafs), "sampled_pairs": len(pairs)})
    print()
    print("N=%d L=%d: GPU %.2f s for 16 score matrices (with host copies), oracle %.1f s" % (N, L, gpu_s, oracle_s))
    for r in rows:
        print(r)
    path = os.environ.get("COVGPU_ERROR_REPORT_DEEP")
    if path:
        with open(path, "w") as f:
            json.dump({"N": N, "L": L, "gpu_seconds": gpu_s, "oracle_seconds": oracle_s, "rows": rows}, f, indent=1)
    assert not bad, bad
    assert erraf <= 1e-12 and errafs <= 1e-12
