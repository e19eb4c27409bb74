"""Benchmark of the covariation path on one synthetic rRNA-scale alignment.

Workload (one step): an N=2,000 x L=3,000 synthetic RNA alignment (coalescent
tree of leaf-to-root length 2.0, 900 planted base pairs in 40 helices of 8-35
pairs, 15% gaps, position-based weights, R-scape's 0.75 gap-column filter),
its 20 null alignments (Fitch ancestors + shuffled substitutions on the same
tree), GTp, MIp, CHIp and RAFp scores with APC for all 21 alignments, the
null histogram and tail fit of each statistic, and the E-values and
E < 0.05 pair list of the input alignment.

  value  column pairs scored per second (21 alignments x L(L-1)/2 pairs per
         step, every pair scored with the four statistics), alignment and
         weights resident on the device, timed with CUDA events on the
         library's stream;
  e2e    the same through the public call with host buffers: the alignment
         and weights copied in and the hit lists copied out in every step.

--impl reference times the reference algorithm on the host cores instead:
R-scape's per-pair counting loop (corr_NaivePP -> mutual_naive_ppij, then
the statistic) and its O(N^2) RAF loop, FP64, on a bounded sample of the
same pairs, one run per statistic as R-scape scores one statistic per run.
That arm never loads the GPU library: its alignment comes from the
generator library alone and the oracle's filter and weights.  Both arms
also report the count+GT rate alone (count_gt_pairs_per_s), the
like-for-like figure without RAF's O(N^2) loop.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np


def pinned_copy(a):
    """A copy of the array in page-locked host memory, so the end-to-end
    host-to-device copies are DMA transfers (the array keeps the pinned
    buffer alive)."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "column-pairs/s (GTp+APC) & E-valued MSAs/s; tensor vs plain GPU at same E<0.05 set"
TYPES = ["GTp", "MIp", "CHIp", "RAFp"]
CFG = dict(N=2000, L=3000, tree_len=2.0, nbp=900, nhelix=40, hmin=8, hmax=35, gap_rate=0.15, gap_mean=3.0,
           seed=42, nshuffle=20)


def load_covgpu():
    import __graft_entry__ as g
    return g._load("covgpu", os.path.join(ROOT, "r-scape_gb300", "covgpu.py"))


def workload(cg):
    c = CFG
    s = cg.Synth(c["N"], c["L"], c["tree_len"], c["nbp"], c["nhelix"], c["hmin"], c["hmax"], c["gap_rate"],
                 c["gap_mean"], seed=c["seed"])
    keep = cg.gapfilter(s.ax, None, 0.75)
    ax = np.ascontiguousarray(s.ax[:, keep])
    w = cg.weights_pb(ax)
    return s, ax, w


def workload_reference():
    """The same alignment for the CPU reference arm, without the GPU library:
    the generator alone (libcovsynth.so, host code) makes the alignment, and
    the oracle applies R-scape's gap-column filter and position-based
    weights."""
    import ctypes as C
    import importlib.util
    spec = importlib.util.spec_from_file_location("rscape_gb300_build", os.path.join(ROOT, "r-scape_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    lib = C.CDLL(b.SYNTHLIB)
    u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
    i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    lib.covgpu_synth2.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_double, C.c_double, C.c_uint64, u8p, i32p, i32p, i32p, f64p, f64p, i32p]
    c = CFG
    N, L = c["N"], c["L"]
    ax = np.zeros((N, L), dtype=np.uint8)
    tree = [np.zeros(N - 1, dtype=np.int32) for _ in range(3)] + [np.zeros(N - 1) for _ in range(2)]
    ct = np.zeros(L, dtype=np.int32)
    st = lib.covgpu_synth2(N, L, 0, c["tree_len"], c["nbp"], c["nhelix"], c["hmin"], c["hmax"], c["gap_rate"],
                           c["gap_mean"], c["seed"], ax, *tree, ct)
    if st:
        raise ValueError("synthetic alignment: bad sizes (status %d)" % st)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    ax = np.ascontiguousarray(ax[:, O.gapfilter(ax, None, 0.75)])
    return ax, O.weights_pb(ax)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


def profile_traffic(kernel):
    """DRAM bytes per launch of a kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel:
                return float(parts[1])
    except OSError:
        pass
    return None


def simulator_rate(cg, e, s, N, L, nrep):
    """Alignments per second of the P(t) simulator on the workload's tree and
    structure (the planted pairs of the kept columns; nrep replicates per
    call, no gaps), measured after the timed steps."""
    Q4, pi4, Q16, pi16 = cg.synth_model()
    keep = np.flatnonzero(cg.gapfilter(s.ax, None, 0.75))
    new = -np.ones(len(s.ct), dtype=np.int64)
    new[keep] = np.arange(len(keep))
    ct = np.full(L, -1, dtype=np.int32)
    for c_new, c_old in enumerate(keep):
        p = s.ct[c_old]
        if p >= 0 and new[p] >= 0:
            ct[c_new] = new[p]
    e.simulate(s.ld, s.rd, Q4, pi4, Q16, pi16, ct, seed=3, first_slot=1, nrep=nrep)   # warm-up
    reps = 3
    t0 = time.perf_counter()
    for r in range(reps):
        e.simulate(s.ld, s.rd, Q4, pi4, Q16, pi16, ct, seed=3, rep0=r * nrep, first_slot=1, nrep=nrep)
    dt = (time.perf_counter() - t0) / reps
    return {"alignments_per_s": nrep / dt, "ms_per_call": 1000.0 * dt, "alignments_per_call": nrep,
            "codes_GB_per_s": nrep * N * L / dt / 1e9, "N": N, "L": L,
            "note": "host-timed covgpu_simulate calls (P tables, evolution, synchronise)"}


def load_learned_null():
    import __graft_entry__ as g
    return g._load("learned_null", os.path.join(ROOT, "r-scape_gb300", "learned_null.py"))


def ragged_per_family(cg, fams, data, counter, device, workers=4):
    """The families run one call each (covgpu_rscape): `workers` host
    threads each drive one context (its own CUDA stream), made for the
    largest size and resized per family.  Per family the alignment and tree
    go in, R-scape's weights (GSC up to 1000 sequences, else position-based)
    and its null count rule run on the device, GTp with APC, and the hit list
    comes out."""
    import threading
    nfam = len(fams)
    engines = [cg.Engine(2000, 1500, maxslots=21, maxnull=20, device=device) for _ in range(workers)]
    errors = []

    def work(k):
        e = engines[k]
        try:
            for i in range(k, nfam, workers):
                f, s = fams[i], data[i]
                e.resize(f["N"], f["L"])
                e.set_alignment(0, s.ax)
                if f["N"] <= 1000:
                    e.weights_gsc(0, set=True)
                else:
                    e.weights_pb(0, set=True)
                e.set_tree(s.parent, s.left, s.right)
                e.rscape(None, None, ["GTp"], counter=counter)
        except Exception as err:   # reported after the join
            errors.append(err)

    t0 = time.perf_counter()
    th = [threading.Thread(target=work, args=(k,)) for k in range(workers)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    dt = time.perf_counter() - t0    # every call returns after its hit list reached the host
    for e in engines:
        e.close()
    if errors:
        raise errors[0]
    return {"families": nfam, "workers": workers, "seconds": dt, "msas_per_s": nfam / dt}


def ragged_families(cg, nfam, counter, device, compare=200):
    """E-valued MSAs/s over families drawn as the ragged-family workload
    draws them (N ~ U[20,2000], L ~ logU[50,1500], tree length ~ U[0.5,3],
    base-pair fraction ~ U[0.1,0.35]; seeds 1..nfam), all in one call of
    covgpu_rscape_families: every device pass one grouped launch over the
    families, the passes from the nulls to the corrected scores a CUDA graph.
    Per family the alignment and tree go in, R-scape's weights (GSC up to
    1000 sequences, else position-based) and its null count rule run on the
    device, GTp with APC, and the hit list comes out.  Families are
    synthesised before the timed region; one warm-up call (allocation, graph
    capture), then the best of two timed calls.  For comparison the first
    `compare` families also run one call each on four host threads."""
    ln = load_learned_null()
    fams = [ln.draw_family(k) for k in range(1, nfam + 1)]
    data = [ln.make_family(f)[0] for f in fams]
    fl = [dict(ax=s.ax, parent=s.parent, left=s.left, right=s.right) for s in data]
    b = cg.Batch(device=device)
    # the count schedule, tuned on the first families
    tuned = None
    if counter == cg.TENSOR:
        bt, bs, times = b.autotune(fl[:min(200, nfam)], ["GTp"], counter=counter)
        tuned = {"simt_below": bt, "raster_superblock": bs,
                 "seconds": {"%d,%d" % k: v for k, v in sorted(times.items())},
                 "families": min(200, nfam)}
    b.rscape(fl, ["GTp"], counter=counter)
    ts = []
    for _ in range(2):
        t0 = time.perf_counter()
        r = b.rscape(fl, ["GTp"], counter=counter)
        ts.append(time.perf_counter() - t0)
    dev_ms, rest_ms, host_ms, nl, nch = b.timing()
    b.close()
    dt = min(ts)
    pairs = sum((x[0]["nshuffle"] + 1) * f["L"] * (f["L"] - 1) // 2 for x, f in zip(r, fams))
    out = {"families": nfam, "seconds": dt, "msas_per_s": nfam / dt, "column_pairs_per_s": pairs / dt,
           "statistic": "GTp", "nulls": "R-scape rule (20 here)", "counter": "tensor" if counter else "simt",
           "mode": "grouped: one launch per pass over all families, device passes as a CUDA graph",
           "launches": nl, "chunks": nch, "schedule": tuned,
           "device_ms": {"nulls_to_corrected_scores": dev_ms, "histograms_fits_evalues": rest_ms},
           "timing": "host wall clock of one call, host buffers in, hit lists out; best of 2 after a warm-up call"}
    if compare > 0:
        k = min(compare, nfam)
        out["per_family_calls"] = ragged_per_family(cg, fams[:k], data[:k], counter, device)
    return out


def batched_nulls(cg, counter, device, steps=3):
    """One N=500 x L=400 alignment (tree length 1.5, 100 base pairs) with 200
    null alignments on its tree, all scored in one batch (GTp with APC)."""
    s = cg.Synth(500, 400, 1.5, 100, 10, 6, 14, 0.08, seed=7)
    w = cg.weights_pb(s.ax)
    e = cg.Engine(500, 400, maxslots=201, maxnull=200, device=device)
    e.set_tree(s.parent, s.left, s.right)
    e.set_weights(w)
    e.set_alignment(0, s.ax)
    e.rscape(None, None, ["GTp"], nshuffle=200, counter=counter)
    ms = []
    for _ in range(steps):
        e.flush_l2()
        e.rscape(None, None, ["GTp"], nshuffle=200, counter=counter)
        ms.append(e.last_timing()[0][4])
    e.close()
    t = statistics.median(ms)
    return {"N": 500, "L": 400, "nulls": 200, "ms_per_msa": t, "msas_per_s": 1000.0 / t,
            "column_pairs_per_s": 201 * 400 * 399 / 2 / (t / 1000.0), "timing": "CUDA events, device-resident"}


def dropin_flow(cg, e, ax, w, ns):
    """R-scape's own calling sequence through the reference-named entry points
    (rscape_cov.h), as R-scape would run it on this workload with GTp:
    calculate_width_histo on the first null, cov_Calculate in RANSS mode on
    each of the ns nulls merged into the cumulative null histogram, then
    cov_Calculate in GIVSS mode on the alignment (src/R-scape.c:1281-1371,
    1614-1724, 2502).  Timed once in the reference's host-array mode (COV
    filled on the host by every call, pp, nseff, ngap and Eval for the given
    alignment; a null's pp stays on the device) and once in
    device-resident mode; host wall clock, host alignments in, hit list out.
    The null alignments come from the engine before the timed region."""
    import ctypes as C
    import importlib.util
    spec = importlib.util.spec_from_file_location("rscape_abi", os.path.join(ROOT, "r-scape_gb300", "rscape_abi.py"))
    abi = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(abi)
    lib = abi.setup_lib(cg.LIBPATH)
    N, L = ax.shape
    e.make_nulls(CFG["seed"], 0, ns, 1)
    abc = abi.Alphabet(1, 4, 18)
    nulls = [abi.MsaHolder(e.get_alignment(1 + k), w, abc) for k in range(ns)]
    real = abi.MsaHolder(ax, w, abc)
    code = cg.covtype_code("GTp")
    out = {"statistic": "GTp", "nulls": ns,
           "timing": "host wall clock, one flow after a warm-up flow (first_flow_seconds: the warm-up flow, with the "
                     "context's creation and, in host-array mode, the page-locking of the host arrays)"}
    for mode, name in ((0, "host_arrays"), (1, "device_resident")):
        mi = lib.corr_Create(L, N, 0, 8, 50, C.byref(abc), 3)
        mi.contents.device_resident = mode
        errbuf = C.create_string_buffer(256)
        th = abi.Thresh(0, 0.05, 0.0, 0.0)
        rnd = abi.Rand(CFG["seed"])
        dt, nhit, first = None, 0, None
        for rep in range(2):
            data = abi.Data(C.pointer(rnd), 3, None, None, mi, C.pointer(th), 1, 0, abi.RANSS, code, N, -1.0, -10.0,
                            0.05, 1.0, 0.0005, 0, 0.0, 0.0, 0.0, None, 1e-6, 0, C.cast(errbuf, C.c_char_p))
            steps = {}
            t0 = time.perf_counter()
            rl, hl, cum = abi.rscape_flow(lib, mi, nulls, real, data, code, timing=steps)
            dt = time.perf_counter() - t0
            first = dt if first is None else first
            nhit = hl.contents.nhit
            lib.cov_FreeHitList(hl)
            lib.cov_FreeRankList(rl)
            lib.cov_FreeRankList(cum)
        lib.corr_Destroy(mi)
        out[name] = {"seconds": dt, "msas_per_s": 1.0 / dt, "column_pairs_per_s": (ns + 2) * L * (L - 1) / 2 / dt,
                     "hits": nhit, "first_flow_seconds": first,
                     "step_seconds": {k: round(v, 4) for k, v in steps.items()}}
    return out


def cpu_reference(ax, w, budget_s, threads):
    """pairs/s of the reference loops on the host: counting + statistic per
    pair (x3: GTp, MIp, CHIp are three runs) and RAF's O(N^2) loop."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    N, L = ax.shape
    # counting + GT sample: rows from the top of the pair triangle
    t0 = time.time()
    rows, npairs = 1, 0
    while True:
        n, _ = O.faithful_rows(ax, w, 0, rows, threads)
        dt = time.time() - t0
        npairs = n
        if dt > budget_s * 0.3 or rows >= L - 1:
            break
        rows = min(L - 1, rows * 2)
        t0 = time.time()
    t_count = dt / npairs
    t0 = time.time()
    nr = max(threads, 8)
    while True:
        n, _ = O.faithful_raf(ax, nr, threads)
        dt = time.time() - t0
        if dt > budget_s * 0.3 or nr >= 4096:
            break
        nr *= 2
        t0 = time.time()
    t_raf = dt / n
    per_pair = 3 * t_count + t_raf
    sample = ("%d pairs of count+GT (rows 0-%d) and %d pairs of RAF of the %dx%d alignment, %d threads; "
              "per pair = 3 x count+statistic + RAF" % (npairs, rows - 1, n, N, L, threads))
    return 1.0 / per_pair, sample, {"count_stat_s_per_pair": t_count, "raf_s_per_pair": t_raf,
                                    "count_gt_pairs_per_s": 1.0 / t_count}


def guarded(fn, *args, **kw):
    """One of the bench line's extra measurements (measured after the headline
    numbers): its result, or its error as a string in the line, so that a
    failing extra neither hides the headline nor fails silently."""
    try:
        return fn(*args, **kw)
    except Exception as ex:   # reported in the line
        return {"error": "%s: %s" % (type(ex).__name__, ex)}


def max_over_ranks(values, world):
    """Each value's largest over the ranks (the slowest rank's times), by an
    all-reduce on the process group; the values themselves with one rank."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--counter", default="auto", choices=["auto", "simt", "tensor"])
    ap.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of CPU baseline sampling")
    ap.add_argument("--once-sim", action="store_true",
                    help="one call of the P(t) simulator on the workload's tree (for profiler captures)")
    ap.add_argument("--once", action="store_true",
                    help="one covgpu_rscape call of the workload and exit (for profiler captures)")
    ap.add_argument("--schedule", type=int, default=0,
                    help="with --once: count-kernel raster super-block to set before a second call "
                         "(e.g. 32004; profiler captures of that schedule)")
    ap.add_argument("--N", type=int, default=None, help="override N (profiling a smaller case)")
    ap.add_argument("--L", type=int, default=None, help="override L (profiling a smaller case)")
    ap.add_argument("--nshuffle", type=int, default=None, help="override the number of nulls")
    ap.add_argument("--types", default=None, help="comma-separated statistics (default GTp,MIp,CHIp,RAFp)")
    ap.add_argument("--families", type=int, default=1000,
                    help="families of the ragged-family batch timed after the main workload (0: skip)")
    ap.add_argument("--once-families", type=int, default=0,
                    help="only one call of the family batch on this many ragged families (profiler launch lists)")
    ap.add_argument("--family-compare", type=int, default=200,
                    help="families also run one call each on four host threads, for comparison (0: skip)")
    ap.add_argument("--no-extras", action="store_true",
                    help="only the main workload: no CPU baseline, simulator, families or batched nulls "
                         "(for profiler launch lists)")
    args = ap.parse_args()
    if args.N:
        CFG["N"] = args.N
    if args.L:
        CFG["L"] = args.L
        CFG["nbp"] = min(CFG["nbp"], args.L // 4)
        CFG["nhelix"] = max(1, min(CFG["nhelix"], CFG["nbp"] // 8))
        CFG["hmin"] = max(1, min(CFG["hmin"], CFG["nbp"] // CFG["nhelix"]))
    if args.nshuffle is not None:
        CFG["nshuffle"] = args.nshuffle
    if args.types:
        TYPES[:] = args.types.split(",")

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    ns = CFG["nshuffle"]
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        ax, w = workload_reference()
        N, L = ax.shape
        P = L * (L - 1) // 2
        pairs_step = (ns + 1) * P
        vals, cgt = [], []
        for k in range(args.warmup + args.steps):
            v, sample, parts = cpu_reference(ax, w, args.cpu_budget / max(1, args.warmup + args.steps) * 2, threads)
            if k >= args.warmup:
                vals.append(v)
                cgt.append(parts["count_gt_pairs_per_s"])
        value = statistics.median(vals)
        out = {"metric": METRIC, "value": value, "unit": "column-pairs/s", "n_gpus": args.gpus,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * pairs_step / value,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic", "impl": "reference",
               "config": {"workload": "rRNA-scale alignment N=%d x L=%d, %d nulls, %s" % (N, L, ns, ",".join(TYPES)),
                          "N": N, "L": L, "nshuffle": ns, "statistics": TYPES},
               "cpu_baseline": {"value": value, "unit": "column-pairs/s", "cores": threads, "kind": "port",
                                "sample": sample, "count_gt_pairs_per_s": statistics.median(cgt)},
               "e2e": {"value": value, "unit": "column-pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
               "msas_per_s": value / pairs_step}
        print(json.dumps(out))
        return

    cg = load_covgpu()
    if args.once_families > 0:
        # one call of the family batch, nothing else (for profiler launch lists)
        ln = load_learned_null()
        fams = [ln.draw_family(k) for k in range(1, args.once_families + 1)]
        fl = []
        for f in fams:
            sf = ln.make_family(f)[0]
            fl.append(dict(ax=sf.ax, parent=sf.parent, left=sf.left, right=sf.right))
        b = cg.Batch()
        t0 = time.perf_counter()
        b.rscape(fl, ["GTp"], counter=cg.TENSOR)
        dt = time.perf_counter() - t0
        dev_ms, rest_ms, host_ms, nl, nch = b.timing()
        b.close()
        print(json.dumps({"once_families": args.once_families, "seconds": dt, "device_ms": [dev_ms, rest_ms],
                          "launches": nl, "chunks": nch}))
        return
    s, ax, w = workload(cg)
    N, L = ax.shape
    P = L * (L - 1) // 2
    pairs_step = (ns + 1) * P
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    counter = {"auto": 0, "simt": 0, "tensor": 1}[args.counter]
    if args.counter == "auto":
        counter = 1 if os.environ.get("COVGPU_COUNTER", "tensor") == "tensor" else 0
    e = cg.Engine(N, L, maxslots=ns + 1, maxnull=ns, device=local)
    e.set_tree(s.parent, s.left, s.right)
    e.set_weights(w)
    e.set_alignment(0, ax)
    try:
        r = e.rscape(None, None, TYPES, nshuffle=ns, counter=counter)
    except RuntimeError:
        counter = 0      # the tensor counter refuses this shape: plain path
        r = e.rscape(None, None, TYPES, nshuffle=ns, counter=counter)
    if args.once_sim:
        print(json.dumps({"once_sim": True, **simulator_rate(cg, e, s, N, L, ns)}))
        return
    if args.once:
        if args.schedule and counter == 1:
            # the given raster (one autotune candidate: four count launches), then the call again
            e.autotune(ns + 1, candidates=(args.schedule,))
            r = e.rscape(None, None, TYPES, nshuffle=ns, counter=counter)
        ms, n = e.last_timing()
        print(json.dumps({"once": True, "N": N, "L": L, "nshuffle": ns, "types": TYPES, "counter": counter,
                          "device_ms": list(ms), "launches": n, "hits": [len(x["hits"]) for x in r]}))
        return
    kind = "tensor" if counter == 1 else "simt"
    tune = None
    if counter == 1:   # the count kernel's tile schedule, picked on this workload before timing
        best, tms = e.autotune(ns + 1)
        tune = {"raster_superblock": best, "ms": tms}
    for _ in range(args.warmup):
        e.flush_l2()
        e.rscape(None, None, TYPES, nshuffle=ns, counter=counter)

    dev_ms, cnt_ms, nl = [], [], 0
    with ClockSampler(local) as clk:
        if world > 1:
            dist.barrier()
        for _ in range(args.steps):
            e.flush_l2()
            res = e.rscape(None, None, TYPES, nshuffle=ns, counter=counter)
            ms, n = e.last_timing()
            dev_ms.append(ms[4])
            cnt_ms.append(ms[1])
            nl += n
        # end to end: host buffers in (page-locked), hit lists out
        pinned_ax, pinned_w = pinned_copy(ax), pinned_copy(w)
        t0 = time.perf_counter()
        e2e_hits = 0
        for _ in range(args.steps):
            r = e.rscape(pinned_ax, pinned_w, TYPES, nshuffle=ns, counter=counter)
            e2e_hits = sum(len(x["hits"]) for x in r)
        e2e_s = (time.perf_counter() - t0) / args.steps
    step_s = sum(dev_ms) / len(dev_ms) / 1000.0
    step_s, e2e_s = max_over_ranks([step_s, e2e_s], world)
    if rank != 0:
        return
    value = world * pairs_step / step_s
    e2e_value = world * pairs_step / e2e_s
    peaks = measured_peaks()
    peak = peaks.get("bf16_tflops") if peaks else 1900.0
    flop_launch = 32.0 * N * P * (ns + 1)      # algorithmic: 16 cells x one multiply-add per sequence
    cnt_s = sum(cnt_ms) / len(cnt_ms) / 1000.0
    achieved = flop_launch / cnt_s / 1e12
    kname = "k_count_umma" if kind == "tensor" else "k_count_simt"
    traffic = profile_traffic(kname)
    if args.no_extras:
        cpu_v, cpu_sample, sim, fam, bnull, plain = None, "skipped (--no-extras)", None, None, None, None
        cpu_parts, dflow = {}, None
    else:
        plain = None
        if counter == 1:
            # the plain SIMT counting path on the same workload, once: its step
            # time and whether it gives the same E < 0.05 pair lists
            e.flush_l2()
            rs = e.rscape(None, None, TYPES, nshuffle=ns, counter=0)
            ms_s = e.last_timing()[0][4]
            same = all(sorted((h[0], h[1]) for h in a["hits"]) == sorted((h[0], h[1]) for h in b["hits"])
                       for a, b in zip(res, rs))
            plain = {"counter": "simt", "ms_per_step": ms_s, "value": pairs_step / (ms_s / 1000.0),
                     "tensor_speedup": ms_s / (step_s * 1000.0), "same_pair_sets": same,
                     "pairs_e_lt_thresh": [len(x["hits"]) for x in rs]}
        cpu_v, cpu_sample, cpu_parts = cpu_reference(ax, w, args.cpu_budget, threads)
        sim = guarded(simulator_rate, cg, e, s, N, L, ns)
        fam = guarded(ragged_families, cg, args.families, counter, local, args.family_compare) \
            if args.families > 0 else None
        bnull = guarded(batched_nulls, cg, counter, local)
        dflow = guarded(dropin_flow, cg, e, ax, w, ns)
    out = {
        "metric": METRIC, "value": value, "unit": "column-pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * step_s, "higher_is_better": True, "scaling": "weak",
        # counts: three FP16 weight limbs (33-bit weights at this N) and the FP8 one-hot on the tensor
        # cores (the SIMT path: the same limbs as FP32), exact integer sums in FP32 combined into
        # double-float counts; statistics in double-float (FP32 pairs) with FP64 means and tables
        "vs_baseline": None, "dtype": ("f32-limbs+df32+f64" if kind == "simt" else "f16x3-limbs+e4m3+df32+f64"),
        "data": "synthetic",
        "config": {"workload": "rRNA-scale alignment N=%d x L=%d, %d nulls, %s" % (N, L, ns, ",".join(TYPES)),
                   "N": N, "L": L, "nshuffle": ns, "statistics": TYPES, "counter": kind,
                   "l2": "flushed (256 MB write) before every step; double-float count tensors "
                         "%.1f GB per step" % ((ns + 1) * (L // 32 + 1) * (L // 32 + 2) / 2 * 1024 * 16 * 8 / 1e9)},
        "msas_per_s": world / step_s,
        "e2e": {"value": e2e_value, "unit": "column-pairs/s", "h2d_bytes_per_step": int(ax.nbytes + w.nbytes),
                "d2h_bytes_per_step": int(e2e_hits * 36 + 4 * 200), "msas_per_s": world / e2e_s},
        "gpu_launches": nl,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic, "kernel": kname,
                     # three FP16 weight limbs: the tensor cores execute 3 x the algorithmic FLOP
                     "executed_frac": (3.0 * achieved / peak) if kind == "tensor" else None,
                     "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if peaks else "fallback 1.9 PFLOP/s"},
        "cpu_baseline": {"value": cpu_v, "unit": "column-pairs/s", "cores": threads, "kind": "port",
                         "sample": cpu_sample,
                         "count_gt_pairs_per_s": cpu_parts["count_gt_pairs_per_s"] if cpu_v else None},
        "hits": [len(x["hits"]) for x in res],
        "simulator": sim,
        "plain_gpu": plain,
        "autotune": tune,
        "ragged_families": fam,
        "batched_nulls": bnull,
        "dropin_flow": dflow,
        "clocks": clk.summary(),
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
