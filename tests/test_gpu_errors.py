"""Largest error of every statistic against the FP64 oracle (needs a GB300).

For each statistic (raw, APC and ASC), unit and float weights, and both
counting paths, prints the maximum absolute error, the maximum relative
error over the pairs whose score is at least 1e-3 of the largest, and the
largest error below that floor in units of the largest score.  With
COVGPU_ERROR_REPORT set to a path the table is also written there as JSON.
The test holds the bound of the parity tests (parity_tol): 1e-5 relative at
or above the floor, 1e-8 of the largest score below it.
"""
import json
import os

import numpy as np
import pytest

from parity_tol import stat_close

pytestmark = pytest.mark.gpu

STATS = ["CHI", "GT", "MI", "MIr", "MIg", "OMES", "RAF", "RAFS", "CCF"]
N, L = 300, 200


def make(covgpu, unit):
    s = covgpu.Synth(N, L, 1.5, 30, 4, 4, 10, 0.1, seed=21, tree_kind=1)
    w = np.ones(N) if unit else covgpu.weights_pb(s.ax) * np.random.default_rng(21).uniform(0.7, 1.3, N)
    return s, w


def test_error_table(covgpu, oracle):
    rows = []
    iu = np.triu_indices(L, 1)
    for counter, cname in [(covgpu.TENSOR, "tensor"), (covgpu.SIMT, "simt")]:
        for unit in (True, False):
            s, w = make(covgpu, unit)
            e = covgpu.Engine(N, L)
            e.set_weights(w)
            e.set_alignment(0, s.ax)
            for corr in ("", "p", "a"):
                for k in range(0, len(STATS), 4):
                    types = [t + corr for t in STATS[k:k + 4]]
                    e.score(types, counter=counter)
                    for q, t in enumerate(types):
                        ref = oracle.cov_calculate(t, s.ax, w)[0][iu]
                        got = e.get_cov(0, q)[iu]
                        ok, rel, small = stat_close(got, ref)
                        rows.append({"stat": t, "weights": "unit" if unit else "float", "counter": cname,
                                     "max_abs": float(np.abs(got - ref).max()), "max_rel": rel,
                                     "small_over_max": small, "ok": ok})
            e.close()
    print()
    print("%-6s %-6s %-7s %12s %12s %12s" % ("stat", "w", "counter", "max abs", "max rel", "small/max"))
    for r in rows:
        print("%-6s %-6s %-7s %12.3e %12.3e %12.3e" % (r["stat"], r["weights"], r["counter"], r["max_abs"],
                                                       r["max_rel"], r["small_over_max"]))
    path = os.environ.get("COVGPU_ERROR_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump({"N": N, "L": L, "rows": rows}, f, indent=1)
    assert all(r["ok"] for r in rows), [r for r in rows if not r["ok"]]
