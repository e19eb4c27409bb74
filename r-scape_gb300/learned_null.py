"""Learned null: training data, training and evaluation.

R-scape takes the null score tail of an alignment from simulated null
alignments (null_rscape, src/R-scape.c:1614-1724; the gamma tail fit of
cov_NullFitGamma, src/covariation.c:1943-1973).  Here a network maps 64
features (covgpu_learned_features: the alignment's summary and the score
summary of a few quick nulls) to the tail that many nulls give, so
alignments inside the training range need only the quick nulls
(covgpu_rscape_learned).

Families are drawn as the ragged-family benchmark draws them: N uniform on
[20, 2000], L log-uniform on [50, 1500], tree length uniform on [0.5, 3],
base-pair fraction uniform on [0.1, 0.35].  Each family is labelled with
the gamma tail fitted to its simulated nulls (GTp with APC), as a correction
of the tail fitted to its quick nulls: ((mu - mu_q)/m_q, log m - log m_q,
log tau - log tau_q), m = tau/lambda the tail's mean excess.  Everything runs on the device through
covgpu; nothing here computes scores on the host.

    python learned_null.py gen   --first 100001 --count 2000 --nnull 200 --nquick 10 --out data.npz
    python learned_null.py train --data data.npz --out net.npz
    python learned_null.py eval  --net net.npz --first 200001 --count 100 --nnull 200 --nquick 10
"""
import argparse
import importlib.util
import json
import math
import os
import sys
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))


def _covgpu():
    if "covgpu" in sys.modules:
        return sys.modules["covgpu"]
    spec = importlib.util.spec_from_file_location("covgpu", os.path.join(_HERE, "covgpu.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["covgpu"] = mod
    spec.loader.exec_module(mod)
    return mod


def draw_family(seed):
    """Sizes and model of one family: N ~ U[20,2000], L ~ logU[50,1500],
    tree length ~ U[0.5,3], base-pair fraction ~ U[0.1,0.35]."""
    rng = np.random.default_rng(seed)
    N = int(rng.integers(20, 2001))
    L = int(round(math.exp(rng.uniform(math.log(50), math.log(1500)))))
    tree_len = float(rng.uniform(0.5, 3.0))
    frac = float(rng.uniform(0.1, 0.35))
    nbp = max(1, int(round(frac * L / 2)))
    hmax = 12
    nhelix = max(1, -(-nbp // 8))
    hmin = min(4, nbp // nhelix)
    return dict(seed=int(seed), N=N, L=L, tree_len=tree_len, bp_frac=frac, nbp=nbp, nhelix=nhelix, hmin=hmin,
                hmax=hmax, gap_rate=0.08, gap_mean=3.0)


def tree_depth(parent, left, right, ld, rd):
    """Mean root-to-leaf length of an Easel-convention tree (node 0 root)."""
    n = len(left)
    depth = np.zeros(n)
    leaf = []
    for v in range(n):   # parent[v] < v: depths are final when v is reached
        for c, b in ((left[v], ld[v]), (right[v], rd[v])):
            if c > 0:
                depth[c] = depth[v] + b
            else:
                leaf.append(depth[v] + b)
    return float(np.mean(leaf))


def make_family(fam):
    cg = _covgpu()
    s = cg.Synth(fam["N"], fam["L"], fam["tree_len"], fam["nbp"], fam["nhelix"], fam["hmin"], fam["hmax"],
                 fam["gap_rate"], fam["gap_mean"], seed=fam["seed"])
    return s, tree_depth(s.parent, s.left, s.right, s.ld, s.rd)


class FamilyRun:
    """One family on the device: alignment, R-scape's weights (GSC up to
    1000 sequences, else position-based; src/R-scape.c:1555-1556), tree."""

    def __init__(self, fam, nnull):
        cg = _covgpu()
        self.fam = fam
        self.s, self.tdepth = make_family(fam)
        self.e = cg.Engine(fam["N"], fam["L"], maxslots=nnull + 1, maxnull=nnull)
        self.e.set_tree(self.s.parent, self.s.left, self.s.right)
        self.e.set_alignment(0, self.s.ax)
        self.w = self.e.weights_gsc(0, set=True) if fam["N"] <= 1000 else self.e.weights_pb(0, set=True)

    def features(self, nquick):
        return self.e.learned_features(self.tdepth, nquick=nquick, counter=_covgpu().TENSOR)

    def full(self, nnull, thresh=0.05, hitcap=1 << 16):
        return self.e.rscape(None, None, ["GTp"], hitcap=hitcap, nshuffle=nnull, thresh=thresh,
                             counter=_covgpu().TENSOR)[0]

    def learned(self, net, nquick, thresh=0.05, hitcap=1 << 16, nnull_fallback=200):
        return self.e.rscape_learned(None, None, net, self.tdepth, "GTp", nquick=nquick, hitcap=hitcap,
                                     nshuffle=nnull_fallback, thresh=thresh, counter=_covgpu().TENSOR)

    def close(self):
        self.e.close()


def relative_summary(X):
    """Quick-null features stored as absolute scores (mean 48, quantiles 50-59,
    maximum 63; deviation 49) re-expressed as covgpu_learned_features gives
    them: offsets from mu_q (60) in units of m_q = exp(61)."""
    X = np.array(X, dtype=np.float64)
    mq, m = X[:, 60:61], np.exp(X[:, 61:62])
    X[:, 48:49] = (X[:, 48:49] - mq) / m
    X[:, 49:50] = X[:, 49:50] / m
    X[:, 50:60] = (X[:, 50:60] - mq) / m
    X[:, 63:64] = (X[:, 63:64] - mq) / m
    return X.astype(np.float32)


def load_training_data(paths, absolute_summary=False):
    """Features, targets and number of quick nulls of generated families.
    Files written before the engine gave the quick-null summary as offsets
    carry no summary="relative" entry; those (or all, with absolute_summary)
    are converted by relative_summary.  ValueError when the files mix
    numbers of quick nulls or name none."""
    zs = [np.load(p) for p in paths]
    Xs = []
    for z in zs:
        rel = "summary" in z and str(z["summary"]) == "relative"
        Xs.append(z["X"] if (rel and not absolute_summary) else relative_summary(z["X"]))
    nq = {int(z["nquick"]) for z in zs if "nquick" in z}
    if len(nq) != 1:
        raise ValueError("training files mix numbers of quick nulls: %s" % sorted(nq))
    return np.concatenate(Xs), np.concatenate([z["T"] for z in zs]), nq.pop()


def tail_of(r):
    """(mu, log(tau/lambda), log tau) of a gamma tail fit, or None."""
    lam, tau = r["lambda_"], r["tau"]
    if r["status"] != 0 or not (lam > 0 and np.isfinite(lam)) or not (tau > 0 and np.isfinite(tau)):
        return None
    return np.array([r["mu"], math.log(tau / lam), math.log(tau)], dtype=np.float64)


def target_of(tail, feat):
    """The network's target: the tail of many nulls relative to the quick
    nulls' fit (features 60-62), as covgpu_rscape_learned reads it back."""
    mq, lmq, ltq = float(feat[60]), float(feat[61]), float(feat[62])
    return np.array([(tail[0] - mq) / math.exp(lmq), tail[1] - lmq, tail[2] - ltq], dtype=np.float32)


def generate(first, count, nnull, nquick=10, log=None):
    """Features X [n][64] (with nquick quick nulls), targets T [n][3] from
    nnull nulls, and family records."""
    X, T, meta = [], [], []
    t0 = time.time()
    for k in range(count):
        fam = draw_family(first + k)
        try:
            run = FamilyRun(fam, nnull)
        except RuntimeError as err:      # e.g. no device memory left for this family's context
            if log:
                print("family %d skipped: %s" % (fam["seed"], err), file=log, flush=True)
            continue
        try:
            f = run.features(nquick)
            r = run.full(nnull)
            tail = tail_of(r)
        finally:
            run.close()
        if tail is None or not np.all(np.isfinite(f)):
            continue
        t = target_of(tail, f)
        if not np.all(np.isfinite(t)):
            continue
        X.append(f)
        T.append(t)
        meta.append([fam["seed"], fam["N"], fam["L"], fam["tree_len"], fam["bp_frac"], r["w"], r["newmass"],
                     tail[0], tail[1], tail[2]])
        if log and (k + 1) % 50 == 0:
            print("gen %d/%d  %.1f s" % (k + 1, count, time.time() - t0), file=log, flush=True)
    return np.array(X, np.float32), np.array(T, np.float32), np.array(meta)


def norm_of(X, T, margin=0.02):
    """Standardisation and the training range (min/max widened by margin of the span)."""
    xm, xs = X.mean(0), X.std(0)
    xs = np.where(xs > 1e-6, xs, 1.0)
    ym, ys = T.mean(0), T.std(0)
    ys = np.where(ys > 1e-6, ys, 1.0)
    lo, hi = X.min(0), X.max(0)
    span = np.maximum(hi - lo, 1e-6)
    return [a.astype(np.float32) for a in (xm, xs, ym, ys, lo - margin * span, hi + margin * span)]


def train(X, T, epochs=300, batch=256, lr=2e-3, wd=1e-4, seed=1, log=None):
    cg = _covgpu()
    net = cg.MLP(batch_cap=max(batch, 512), seed=seed)
    net.set_norm(*norm_of(X, T))
    t0 = time.time()
    hist = net.train(X, T, epochs, batch=batch, lr=lr, wd=wd, seed=seed)
    if log:
        print("train: %d rows, %d epochs, %.2f s, loss %.4f -> %.4f" % (len(X), epochs, time.time() - t0, hist[0],
                                                                        hist[-1]), file=log, flush=True)
    return net, hist


def val_loss(net, X, T):
    """Mean squared error on standardised targets."""
    ym, ys = net.norm()[2:4]
    return float(np.mean(((net.forward(X) - T) / ys) ** 2))


def train_selected(X, T, grid_epochs=(5, 10, 20, 40, 80, 160), grid_wd=(1e-4, 1e-2, 1e-1, 0.3, 1.0), val_frac=0.15,
                   batch=256, lr=2e-3, seed=1, log=None):
    """Epochs and weight decay chosen on a held-out split of the families;
    the network kept is trained with the chosen setting on every family."""
    rng = np.random.default_rng(seed)
    idx = rng.permutation(len(X))
    nv = max(1, int(val_frac * len(X)))
    va, tr = idx[:nv], idx[nv:]
    best = None
    for wd in grid_wd:
        for ep in grid_epochs:
            net, hist = train(X[tr], T[tr], epochs=ep, batch=batch, lr=lr, wd=wd, seed=seed)
            v = val_loss(net, X[va], T[va])
            if log:
                print("select: wd %g epochs %d train %.4f val %.4f" % (wd, ep, hist[-1], v), file=log, flush=True)
            if best is None or v < best[0]:
                if best is not None:
                    best[1].close()
                best = (v, net, ep, wd)
            else:
                net.close()
    zero = float(np.mean(((T[va] - T[tr].mean(0)) / T[tr].std(0)) ** 2))
    best[1].close()
    net, _ = train(X, T, epochs=best[2], batch=batch, lr=lr, wd=best[3], seed=seed, log=log)
    return net, dict(val_loss=best[0], epochs=best[2], wd=best[3], val_loss_mean_predictor=zero,
                     train_rows=len(X), val_rows=len(va))


def train_members(X, T, n, epochs, wd, batch=256, lr=2e-3, seed=1, log=None):
    """n networks with the same setting on every family, seeds seed..seed+n-1
    (one standardisation, that of the data)"""
    return [train(X, T, epochs=epochs, batch=batch, lr=lr, wd=wd, seed=seed + k, log=log)[0] for k in range(n)]


def save(net, path, nquick, members=None):
    """The network's standardisation and parameters; with members (networks
    trained on the same standardisation) params holds one row per member."""
    xm, xs, ym, ys, lo, hi = net.norm()
    params = np.stack([m.params() for m in members]) if members else net.params()
    np.savez_compressed(path, params=params, xmean=xm, xstd=xs, ymean=ym, ystd=ys, xlo=lo, xhi=hi,
                        nquick=np.int32(nquick))


def load(path, batch_cap=512):
    """A saved network; a file with several parameter rows is an ensemble
    (covgpu_mlp_set_members), its first row the primary parameters."""
    cg = _covgpu()
    z = np.load(path)
    net = cg.MLP(batch_cap=batch_cap)
    P = np.asarray(z["params"], dtype=np.float32)
    net.set_params(P[0] if P.ndim == 2 else P)
    net.set_norm(z["xmean"], z["xstd"], z["ymean"], z["ystd"], z["xlo"], z["xhi"])
    if P.ndim == 2 and len(P) > 1:
        net.set_members(P)
    return net


def mean_predictor(net):
    """The method without the network: every alignment gets the training
    set's mean tail (all weights zero, same standardisation and range)."""
    cg = _covgpu()
    m = cg.MLP(batch_cap=8)
    m.set_params(np.zeros(cg.NPARAM, np.float32))
    xm, xs, ym, ys, lo, hi = net.norm()
    m.set_norm(xm, xs, ym, ys, lo, hi)
    return m


def evalue_errors(truth, other, ecut=1.0):
    """Relative E-value errors over the pairs with true E < ecut (pairs the
    other method leaves above its listing threshold count as missing), and
    the agreement of the E < 0.05 sets (|A and B| / |A or B|, 1 when both are
    empty)."""
    t = {(i, j): E for (i, j, sc, E, p) in truth["hits"] if E < ecut}
    o = {(i, j): E for (i, j, sc, E, p) in other["hits"]}
    errs = [abs(o[k] - E) / E if k in o else float("inf") for k, E in t.items()]
    A = {k for k, E in t.items() if E < 0.05}
    B = {k for k, E in o.items() if E < 0.05}
    agree = 1.0 if not (A | B) else len(A & B) / len(A | B)
    return errs, agree, len(A), len(B)


def evaluate(net, first, count, nnull, nquick=10, few=20, log=None):
    """Held-out families against the fit from nnull simulated nulls: the
    learned null (nquick quick nulls), the same quick nulls fitted without
    the network, the training set's mean tail, and a few-null fit."""
    base = mean_predictor(net)
    rows = []
    for k in range(count):
        fam = draw_family(first + k)
        run = FamilyRun(fam, nnull)
        try:
            truth = run.full(nnull, thresh=1.0, hitcap=1 << 20)
            if tail_of(truth) is None:
                continue
            lr, used = run.learned(net, nquick, thresh=10.0, hitcap=1 << 20, nnull_fallback=nnull)
            mr, mused = run.learned(base, nquick, thresh=10.0, hitcap=1 << 20, nnull_fallback=nnull)
            qr = run.full(nquick, thresh=10.0, hitcap=1 << 20)
            fr = run.full(few, thresh=10.0, hitcap=1 << 20) if few else None
        finally:
            run.close()
        ntail = sum(1 for h in truth["hits"] if h[3] < 1.0)
        row = dict(seed=fam["seed"], N=fam["N"], L=fam["L"], used_net=used, ntrue=0, ntail=ntail)
        for name, r in (("net", lr), ("mean", mr), ("quick", qr), ("few", fr)):
            if r is None:
                continue
            errs, agree, na, nb = evalue_errors(truth, r)
            row[name + "_med"] = float(np.median(errs)) if errs else 0.0
            row[name + "_p90"] = float(np.percentile(errs, 90)) if errs else 0.0
            row[name + "_agree"] = agree
            row[name + "_nsig"] = nb
            row["ntrue"] = na
        row["sim_nulls"] = nquick if used else nquick + nnull
        rows.append(row)
        if log and (k + 1) % 10 == 0:
            print("eval %d/%d" % (k + 1, count), file=log, flush=True)
    base.close()
    return rows


def summarize(rows, nnull):
    """Medians over the families the network handled that have at least one
    pair with true E < 1 (the others have no tail to compare); pair-set
    agreement over the families where either method finds an E < 0.05 pair."""
    used = [r for r in rows if r["used_net"]]
    tail = [r for r in used if r["ntail"] > 0]
    sims = sum(r["sim_nulls"] for r in rows)
    out = dict(families=len(rows), used_net=len(used), fallback=len(rows) - len(used),
               families_with_tail=len(tail), simulated_nulls=sims, full_nulls=nnull * len(rows),
               null_reduction=(nnull * len(rows) / sims) if sims else float("inf"))
    for name in ("net", "mean", "quick", "few"):
        v = [r[name + "_med"] for r in tail if name + "_med" in r]
        if not v:
            continue
        fin = [x for x in v if np.isfinite(x)]
        out[name + "_median_rel_E_error"] = float(np.median(v))
        out[name + "_p75_rel_E_error"] = float(np.percentile(fin, 75)) if fin else float("nan")
        out[name + "_finite_frac"] = len(fin) / len(v)
        ag = [r[name + "_agree"] for r in used if r["ntrue"] > 0 or r.get(name + "_nsig", 0) > 0]
        out[name + "_pairset_agreement_mean"] = float(np.mean(ag)) if ag else 1.0
    out["net_better_than_quick"] = sum(1 for r in tail if r["net_med"] < r["quick_med"])
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="cmd", required=True)
    g = sub.add_parser("gen")
    g.add_argument("--first", type=int, default=100001)
    g.add_argument("--count", type=int, default=1000)
    g.add_argument("--nnull", type=int, default=200)
    g.add_argument("--nquick", type=int, default=10)
    g.add_argument("--out", required=True)
    t = sub.add_parser("train")
    t.add_argument("--data", nargs="+", required=True)
    t.add_argument("--batch", type=int, default=256)
    t.add_argument("--absolute-summary", action="store_true",
                   help="treat every data file as holding the quick-null summary as absolute scores")
    t.add_argument("--lr", type=float, default=2e-3)
    t.add_argument("--members", type=int, default=1,
                   help="train this many networks (seeds 1..) with the selected setting and save them as an ensemble")
    t.add_argument("--out", required=True)
    e = sub.add_parser("eval")
    e.add_argument("--net", required=True)
    e.add_argument("--first", type=int, default=200001)
    e.add_argument("--count", type=int, default=100)
    e.add_argument("--nnull", type=int, default=200)
    e.add_argument("--nquick", type=int, default=10)
    e.add_argument("--few", type=int, default=20)
    e.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    if a.cmd == "gen":
        X, T, meta = generate(a.first, a.count, a.nnull, nquick=a.nquick, log=sys.stderr)
        np.savez_compressed(a.out, X=X, T=T, meta=meta, nnull=a.nnull, nquick=a.nquick, summary="relative")
        print(json.dumps(dict(rows=len(X), out=a.out)))
    elif a.cmd == "train":
        try:
            X, T, nquick = load_training_data(a.data, absolute_summary=a.absolute_summary)
        except ValueError as e:
            raise SystemExit(str(e))
        net, info = train_selected(X, T, batch=a.batch, lr=a.lr, log=sys.stderr)
        members = None
        if a.members > 1:
            members = [net] + train_members(X, T, a.members - 1, info["epochs"], info["wd"], batch=a.batch,
                                            lr=a.lr, seed=2, log=sys.stderr)
        save(net, a.out, nquick, members)
        print(json.dumps(dict(rows=len(X), members=a.members, **info)))
    else:
        net = load(a.net)
        rows = evaluate(net, a.first, a.count, a.nnull, nquick=a.nquick, few=a.few, log=sys.stderr)
        s = summarize(rows, a.nnull)
        if a.out:
            with open(a.out, "w") as f:
                json.dump(dict(summary=s, rows=rows), f, indent=1)
        print(json.dumps(s))


if __name__ == "__main__":
    main()
