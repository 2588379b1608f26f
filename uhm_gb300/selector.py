"""Learned per-front precision selector: training data, labels, training, evaluation.

The network itself (12 -> 64 -> 64 -> 3, hand-written CUDA training and
inference kernels) lives in ``csrc/k_selector.cu``; the features are computed
by the engine from the element matrices and the tree
(``Mesh.front_features``).  This module produces the labels and drives the
training:

* Instances: 3D heterogeneous diffusion on n^3 hex meshes (n = 8, 12, 16;
  ``SIZES``), per-element order p ~ U{p_lo..p_hi}, lognormal coefficient (sigma = 2)
  clipped to a contrast C ~ 10^U(0, 6).  Half of the n = 8 instances also
  carry a negative reaction term c = -s * lambda_min (s = 1 - 10^-U(1, 5.5)),
  which moves the operator towards its first eigenvalue; without such
  instances every front would always take the cheapest precision.
* Labels are generated by the solver: a ladder of per-front precision
  assignments (by depth below the root) is solved with at most ``k``
  refinement steps; among the assignments that reach the backward-error
  target without the FP64 redo, the fastest (ties within 5 % go to the lower
  precision) gives every front its label.
* Training runs on the GPU through ``api.mlp_train`` (Adam, class-weighted
  cross-entropy) on a level-balanced sample (every tree level of every
  instance weighs alike); the weights ship as ``selector_weights.npz``.
* At run time the engine decodes the per-front probabilities per tree level
  (FP64 only when confident) and redoes a missed solve in FP64.

    python -m uhm_gb300.selector --out DIR [--train 400 --test 112]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time
from dataclasses import asdict, dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "selector_weights.npz")
CLASS_PREC = (0, 1, 2)          # class -> engine precision: FP64, FP32, BF16X3
TOL = 1e-12
K_STEPS = 3


# ----------------------------------------------------------------------------
# parameters
# ----------------------------------------------------------------------------
def init_params(seed: int = 0) -> np.ndarray:
    """He-uniform weights, zero biases, in the kernel's packed layout."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((12, 64), (64, 64), (64, 3)):
        lim = math.sqrt(6.0 / fan_in)
        parts.append(rng.uniform(-lim, lim, size=fan_out * fan_in))
        parts.append(np.zeros(fan_out))
    return np.concatenate(parts).astype(np.float32)


def load_weights(path: str = WEIGHTS):
    if not os.path.exists(path):
        return None
    with np.load(path) as d:
        return d["params"].astype(np.float32)


def save_weights(params, path: str = WEIGHTS, meta: dict | None = None) -> None:
    np.savez(path, params=np.asarray(params, np.float32), meta=json.dumps(meta or {}))


# ----------------------------------------------------------------------------
# instances
# ----------------------------------------------------------------------------
@dataclass
class Instance:
    seed: int
    n: int
    p_lo: int
    p_hi: int
    contrast: float
    shift: float          # s in [0, 1): reaction c = -s * lambda_min
    lam: float = 0.0      # lambda_min of the unshifted operator (filled when shift > 0)


# mesh sizes of the training mix: (n, p_lo, p_hi, share, shifted instances allowed)
SIZES = ((8, 2, 5, 0.5, True), (12, 2, 5, 0.2, False), (16, 2, 4, 0.1, False), (16, 4, 4, 0.1, False),
         (16, 3, 5, 0.1, False))


def sample_instances(count: int, seed: int, sizes=SIZES):
    """Instances of the training mix; the shifted ones only on the smallest
    meshes, where lambda_min is cheap to compute."""
    rng = np.random.default_rng(seed)
    shares = np.array([sz[3] for sz in sizes], dtype=np.float64)
    out = []
    for i in range(count):
        n, p_lo, p_hi, _, shiftable = sizes[int(rng.choice(len(sizes), p=shares / shares.sum()))]
        c = float(10.0 ** rng.uniform(0.0, 6.0))
        s = 0.0
        if shiftable and rng.random() < 0.5:
            s = float(1.0 - 10.0 ** (-rng.uniform(1.0, 5.5)))
        out.append(Instance(seed=int(seed * 100003 + i), n=n, p_lo=p_lo, p_hi=p_hi, contrast=c, shift=s))
    return out


def _fields(inst: Instance):
    rng = np.random.default_rng(inst.seed)
    ne = inst.n ** 3
    p = rng.integers(inst.p_lo, inst.p_hi + 1, ne)
    lk = 2.0 * rng.standard_normal(ne)
    c = 0.5 * math.log(inst.contrast)
    kappa = np.exp(np.clip(lk, -c, c))
    return p, kappa


def make_mesh(inst: Instance):
    from . import hpfem
    p, kappa = _fields(inst)
    react = None
    if inst.shift > 0:
        react = -inst.shift * inst.lam * np.ones(inst.n ** 3)
    return hpfem.build_mesh(3, inst.n, p, kappa=kappa, react=react, seed=inst.seed)


def assemble_sparse(spec):
    """Assembled operator sum_e P_e^T A_e P_e (scipy CSR)."""
    import scipy.sparse as sp
    off = np.concatenate([[0], np.cumsum(spec.node_ndof)]).astype(np.int64)
    rows, cols, vals = [], [], []
    for e in range(spec.n_leaves):
        d = np.concatenate([np.arange(off[nd], off[nd] + spec.node_ndof[nd]) for nd in spec.element_nodes(e)]
                           + [np.zeros(0, np.int64)]).astype(np.int64)
        if d.size == 0:
            continue
        A = spec.element_matrix(e)
        rows.append(np.repeat(d, d.size))
        cols.append(np.tile(d, d.size))
        vals.append(A.ravel(order="C"))
    n = int(off[-1])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def lambda_min(inst: Instance) -> float:
    """Smallest generalized eigenvalue of (K, M) for the instance's p and kappa."""
    import scipy.sparse.linalg as sla
    from . import hpfem
    p, kappa = _fields(inst)
    K = assemble_sparse(hpfem.build_mesh(3, inst.n, p, kappa=kappa, seed=inst.seed))
    M = assemble_sparse(hpfem.build_mesh(3, inst.n, p, kappa=np.zeros(inst.n ** 3),
                                         react=np.ones(inst.n ** 3), seed=inst.seed))
    return float(sla.eigsh(K.tocsc(), k=1, M=M.tocsc(), sigma=0, which="LM", return_eigenvectors=False)[0])


def _lambda_worker(d):
    return lambda_min(Instance(**d))


def fill_lambdas(insts, workers: int = 0):
    """lambda_min for the shifted instances, in a spawn-started process pool."""
    todo = [i for i in insts if i.shift > 0]
    if not todo:
        return
    if workers <= 1:
        for i in todo:
            i.lam = lambda_min(i)
        return
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(workers) as pool:
        lams = pool.map(_lambda_worker, [asdict(i) for i in todo], chunksize=1)
    for i, lam in zip(todo, lams):
        i.lam = lam


# ----------------------------------------------------------------------------
# labels
# ----------------------------------------------------------------------------
# (name, class of the fronts at depth < top, class of the others)
LADDER = [("bf16", 0, None, 2), ("fp32@top1", 1, 1, 2), ("fp32@top2", 2, 1, 2), ("fp32", 0, None, 1),
          ("fp64@top1", 1, 0, 1), ("fp64@top2", 2, 0, 1), ("fp64@top3", 3, 0, 1), ("fp64", 0, None, 0)]


def ladder_classes(rung, depth):
    _, top, top_cls, rest = rung
    cls = np.full(depth.shape, rest, np.int32)
    if top_cls is not None:
        cls[depth < top] = top_cls
    return cls


def front_depth(m):
    eid, gen, fs, ss = m.fronts()
    return eid, gen - gen.min()


def run_assignment(m, n_el, eid, cls, k=K_STEPS, reps=2):
    """Factor + solve with per-front classes; time of the last repetition."""
    from . import api
    pr = -np.ones(n_el, np.int32)
    pr[eid] = np.asarray(CLASS_PREC, np.int32)[cls]
    m.set_mode(1, api.PREC_BF16X3, TOL, k)
    m.set_front_precision(pr)
    rec = None
    for r in range(reps):
        m.chol_with_free()
        m.solve_chol()
        t = m.timing()
        st = m.status()
        rec = dict(ms=t["factor_ms"] + t["solve_ms"] + t["refine_ms"], it=int(t["ir_iters"]),
                   berr=float(t["berr"]), ok=bool(st == 0 and 0 <= t["berr"] <= TOL), status=int(st))
        if not rec["ok"]:
            break
    return rec


def run_policy(m, mode, prec, k=K_STEPS, reps=2):
    from . import api
    m.set_mode(mode, prec, TOL, k)
    m.set_front_precision(-np.ones(1, np.int32))
    rec = None
    for r in range(reps):
        m.chol_with_free()
        m.solve_chol()
        t = m.timing()
        st = m.status()
        berr = float(t["berr"]) if mode == 1 else float(m.backward_error())
        rec = dict(ms=t["factor_ms"] + t["solve_ms"] + t["refine_ms"], it=int(t["ir_iters"]), berr=berr,
                   ok=bool(st == 0 and 0 <= berr <= TOL), status=int(st))
    return rec


N_LOW_RUNGS = 4      # rungs without FP64 fronts (FP64 runs at a small fraction of FP32 speed on this GPU)
TIE = 1.05           # a rung within 5 % of the fastest counts as tied; ties go to the lower precision


def label_instance(m, spec):
    """Features per front and the solver-generated label per front: the
    fastest rung of the ladder that meets the target within K_STEPS refinement
    steps without the FP64 redo; rungs with FP64 fronts are tried only when no
    FP32 / BF16 rung passes."""
    eid, depth = front_depth(m)
    feats = m.front_features()
    results = []
    for j, rung in enumerate(LADDER):
        if j >= N_LOW_RUNGS and any(r["ok"] for r in results):
            break
        cls = ladder_classes(rung, depth)
        rec = run_assignment(m, spec.n_elements, eid, cls)
        rec["rung"] = rung[0]
        results.append(rec)
    passing = [(r["ms"], i) for i, r in enumerate(results) if r["ok"]]
    if passing:
        best_ms = min(ms for ms, _ in passing)
        win = min(i for ms, i in passing if ms <= TIE * best_ms)
    else:
        win = len(LADDER) - 1
    return feats, ladder_classes(LADDER[win], depth), results, win


# ----------------------------------------------------------------------------
# evaluation of a trained selector against the methods without it
# ----------------------------------------------------------------------------
def evaluate_instance(m, spec, params):
    from . import api
    out = {"plain_fp64": run_policy(m, 0, api.PREC_FP64),
           "fixed_bf16": run_policy(m, 1, api.PREC_BF16X3)}
    m.set_selector(params)
    out["learned"] = run_policy(m, 1, api.PREC_LEARNED)
    prec, cls = m.front_precision()
    out["learned"]["classes"] = np.bincount(cls[cls >= 0], minlength=3).tolist()
    return out


def level_balanced(X, Y, G, copies: int = 64, seed: int = 0):
    """Training samples with every tree level of every instance weighted
    alike: a level with m fronts contributes min(m, copies) distinct fronts,
    each repeated max(1, copies // m) times (the root decides most of the
    cost but is one front among thousands of leaves)."""
    rng = np.random.default_rng(seed)
    xs, ys = [], []
    depth = np.round(X[:, 3] * 8).astype(np.int64)
    for g in np.unique(G):
        idx_g = np.where(G == g)[0]
        for d in np.unique(depth[idx_g]):
            idx = idx_g[depth[idx_g] == d]
            if idx.size > copies:
                idx = rng.choice(idx, copies, replace=False)
            rep = max(1, copies // idx.size)
            xs.append(np.repeat(X[idx], rep, axis=0))
            ys.append(np.repeat(Y[idx], rep))
    return np.concatenate(xs).astype(np.float32), np.concatenate(ys).astype(np.int32)


def class_weights(y, power: float = 0.5):
    """(N / N_c)^power per class, normalised to mean 1 over present classes
    (power 1: fully balanced; 0.5: a milder push towards rare classes)."""
    cnt = np.bincount(y, minlength=3).astype(np.float64)
    w = np.where(cnt > 0, (cnt.sum() / (3.0 * np.maximum(cnt, 1.0))) ** power, 0.0)
    return (w / w[cnt > 0].mean()).astype(np.float32)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--train", type=int, default=400)
    ap.add_argument("--test", type=int, default=112)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--level-copies", type=int, default=256)
    ap.add_argument("--class-power", type=float, default=0.5)
    ap.add_argument("--dataset", default=None, help="reuse the labels of an earlier run (its --out folder)")
    ap.add_argument("--no-eval", action="store_true")
    ap.add_argument("--workers", type=int, default=max(1, (os.cpu_count() or 2) - 1))
    args = ap.parse_args(argv)
    os.makedirs(args.out, exist_ok=True)
    t0 = time.time()
    if args.dataset:
        d = np.load(os.path.join(args.dataset, "selector_dataset.npz"))
        with open(os.path.join(args.dataset, "selector_labels.json")) as f:
            rows = json.load(f)
        Xall, Yall, Gall, split = d["X"], d["Y"], d["G"], int(d["split"])
        insts = [Instance(**r["inst"]) for r in rows]
        t_lam = 0.0
        from . import api, build
        build.build()
    else:
        insts = sample_instances(args.train + args.test, args.seed)
        fill_lambdas(insts, args.workers)               # process pool before any GPU call
        t_lam = time.time() - t0
        from . import api, build
        build.build()
        X, Y, G, rows = [], [], [], []
        for j, inst in enumerate(insts):
            spec = make_mesh(inst)
            m = api.load_spec(spec)
            feats, lab, res, win = label_instance(m, spec)
            X.append(feats)
            Y.append(lab)
            G.append(np.full(len(lab), j, np.int32))
            rows.append(dict(inst=asdict(inst), win=LADDER[win][0], results=res))
            del m
        Xall, Yall, Gall, split = np.concatenate(X), np.concatenate(Y), np.concatenate(G), args.train
        with open(os.path.join(args.out, "selector_labels.json"), "w") as f:
            json.dump(rows, f)
        np.savez_compressed(os.path.join(args.out, "selector_dataset.npz"), X=Xall, Y=Yall, G=Gall, split=split)
    tr = Gall < split
    Xtr, Ytr = level_balanced(Xall[tr], Yall[tr], Gall[tr], args.level_copies, args.seed)
    w = class_weights(Ytr, args.class_power)
    params, hist = api.mlp_train(Xtr, Ytr, init_params(args.seed), epochs=args.epochs, batch=1024, lr=2e-3,
                                 seed=args.seed, class_weight=w)
    pred_te, _ = api.mlp_predict(Xall[~tr], params)
    meta = dict(train=int(split), test=int(len(insts) - split), seed=args.seed, sizes=[list(z) for z in SIZES],
                epochs=args.epochs, level_copies=args.level_copies, class_power=args.class_power,
                class_weight=w.tolist(), loss_hist=[float(v) for v in hist],
                test_acc_per_front=float((pred_te == Yall[~tr]).mean()),
                label_counts=np.bincount(Yall[tr], minlength=3).tolist(), t_lambda_s=t_lam)
    save_weights(params, os.path.join(args.out, "selector_weights.npz"), meta)
    if args.no_eval:
        print(json.dumps(meta))
        return
    evals = []
    for j, inst in enumerate(insts[split:]):
        spec = make_mesh(inst)
        m = api.load_spec(spec)
        ev = evaluate_instance(m, spec, params)
        ev["inst"] = asdict(inst)
        ev["best"] = min((r["ms"] for r in rows[split + j]["results"] if r["ok"]), default=None)
        evals.append(ev)
        del m
    from . import hpfem
    spec = hpfem.poisson3d(16, 4, seed=0)           # the benchmark workload
    m = api.load_spec(spec)
    bench_eval = evaluate_instance(m, spec, params)
    del m
    meta["t_total_s"] = time.time() - t0
    with open(os.path.join(args.out, "selector_eval.json"), "w") as f:
        json.dump(dict(meta=meta, evals=evals, poisson3d_16_p4=bench_eval), f)
    summary = summarize(evals, meta)
    summary["poisson3d_16_p4"] = {k: {kk: v[kk] for kk in ("ms", "ok", "it")} for k, v in bench_eval.items()}
    summary["poisson3d_16_p4"]["learned_classes"] = bench_eval["learned"]["classes"]
    print(json.dumps(summary))


def summarize(evals, meta=None):
    def agg(key):
        ms = np.array([e[key]["ms"] for e in evals])
        ok = np.array([e[key]["ok"] for e in evals])
        return dict(mean_ms=float(ms.mean()), ok_frac=float(ok.mean()))
    out = {k: agg(k) for k in ("plain_fp64", "fixed_bf16", "learned")}
    best = [e["best"] for e in evals if e["best"] is not None]
    out["best_mean_ms"] = float(np.mean(best)) if best else None
    out["speedup_learned_vs_plain"] = out["plain_fp64"]["mean_ms"] / out["learned"]["mean_ms"]
    out["speedup_learned_vs_fixed"] = out["fixed_bf16"]["mean_ms"] / out["learned"]["mean_ms"]
    if meta:
        out.update({k: meta[k] for k in ("test_acc_per_front", "label_counts") if k in meta})
    return out


if __name__ == "__main__":
    main()
