"""Measurements of the workloads beside the headline benchmark (one GPU).

``python -m uhm_gb300.measure convdiff``
    3D convection-diffusion, 24^3 hex p=3, lognormal kappa (sigma 2, contrast
    up to 1e4), beta = (1, .5, .25) * 100, nested-dissection merges 3, 2, 2, 2
    (leaves to root; root front 14,911): LU with partial pivoting inside
    each eliminated block (the reference's Mesh_::lu_piv_with_free /
    solve_lu_piv path).  Plain FP64 fronts against FP32 (or, --prec 2,
    BF16-split with tensor-core trailing updates) fronts with FP64
    element-wise refinement to backward error 1e-12; seconds per
    factor+solve(+refine), GFLOP/s over the LAWN-41 count, backward errors.

``python -m uhm_gb300.measure elements``
    Element matrices of 3D Poisson 16^3 hex p=4 generated on the device
    (uhm_gpu_generate_lobatto_elements, recipe upload included) against the
    host mesh build (numpy); also checks that the solution from generated
    matrices has the same bits as from copied-in ones.

``python -m uhm_gb300.measure batch``
    Many independent 3D Poisson meshes (n hexes per side and order p drawn
    uniformly from the given ranges, 16 right-hand sides each) joined into
    forests (hpfem.forest) so that same-generation fronts of all meshes share
    each launch.  Reports solves per second (mesh x right-hand side per
    second) and the per-mesh time distribution for the batched forests and
    for the same meshes solved one at a time.

Every number is taken from the engine's CUDA-event timings of the factor,
solve and refinement phases, after warm-up, with the inputs resident on the
device.
"""
from __future__ import annotations

import argparse
import json
import statistics
import time

import numpy as np

from . import api, hpfem

TOL = 1e-12


def _step(m, method):
    m.factor(method)
    m.solve(method)
    t = m.timing()
    return (t["factor_ms"] + t["solve_ms"] + t["refine_ms"]) * 1e-3, t


def convdiff(n=24, p=3, seed=0, steps=3, warmup=1, plain_steps=1, merges=(3, 2, 2, 2), prec=api.PREC_FP32):
    t0 = time.perf_counter()
    spec = hpfem.convdiff3d(n, p, seed=seed, merges=list(merges) if merges else None)
    t_gen = time.perf_counter() - t0
    m = api.load_spec(spec)
    method = api.UHM_LU_PIV
    fd, _ = m.estimate_cost(method)
    out = {"workload": (f"3D convection-diffusion {n}^3 hex p={p}, merges {list(merges) if merges else 'auto'}, "
                        "LU with partial pivoting, 1 RHS"),
           "n_dof": int(spec.n_dof()), "n_fronts": int(spec.n_elements),
           "factor_gflop_lawn41": fd / 1e9, "mesh_generation_s": t_gen}
    m.set_mode(0)
    for _ in range(warmup):
        _step(m, method)
    pl = [_step(m, method) for _ in range(plain_steps)]
    out["plain_fp64"] = {"s": statistics.median([r[0] for r in pl]),
                         "factor_ms": pl[-1][1]["factor_ms"], "solve_ms": pl[-1][1]["solve_ms"],
                         "backward_error": m.backward_error()}
    out["plain_fp64"]["factor_gflops"] = fd / 1e9 / (pl[-1][1]["factor_ms"] * 1e-3)
    m.set_mode(1, prec, TOL, 10)
    for _ in range(warmup):
        _step(m, method)
    mx = [_step(m, method) for _ in range(steps)]
    last = mx[-1][1]
    key = {api.PREC_FP32: "mixed_fp32_ir", api.PREC_BF16X3: "mixed_bf16x3_ir"}.get(prec, "mixed_ir")
    out["mixed_precision"] = key
    out[key] = {"s": statistics.median([r[0] for r in mx]),
                            "factor_ms": last["factor_ms"], "solve_ms": last["solve_ms"],
                            "refine_ms": last["refine_ms"], "ir_iters": last["ir_iters"],
                            "berr_first_solve": last.get("berr_first"), "backward_error": last["berr"],
                            "status": m.status()}
    out[key]["factor_gflops"] = fd / 1e9 / (last["factor_ms"] * 1e-3)
    out["speedup_mixed_vs_plain"] = out["plain_fp64"]["s"] / out[key]["s"]
    return out


def _group(specs, max_dofs):
    """Consecutive meshes into forests of at most ``max_dofs`` dofs each."""
    groups, cur, acc = [], [], 0
    for s in specs:
        d = s.n_dof()
        if cur and acc + d > max_dofs:
            groups.append(cur)
            cur, acc = [], 0
        cur.append(s)
        acc += d
    if cur:
        groups.append(cur)
    return groups


def batch(n_meshes=64, seed=0, n_range=(8, 12), p_range=(2, 4), n_rhs=16, prec=api.PREC_FP32,
          max_dofs=6_000_000, steps=3, warmup=1, separate=True):
    t0 = time.perf_counter()
    specs = hpfem.batch3d(n_meshes, seed=seed, n_range=n_range, p_range=p_range, n_rhs=n_rhs)
    t_gen = time.perf_counter() - t0
    method = api.UHM_CHOL
    groups = _group(specs, max_dofs)
    out = {"workload": (f"{n_meshes} independent 3D Poisson meshes, n uniform in {list(n_range)}, "
                        f"p uniform in {list(p_range)}, {n_rhs} RHS each"),
           "n_dof_total": int(sum(s.n_dof() for s in specs)), "forests": len(groups),
           "precision": ["fp64", "fp32", "bf16x3", "bf16x6"][prec], "mesh_generation_s": t_gen}
    # batched: one forest per group, its meshes done when the forest is done
    per_mesh, total, berr_worst, iters = [], 0.0, 0.0, []
    for g in groups:
        f = hpfem.forest(g)
        m = api.load_spec(f)
        m.set_mode(1, prec, TOL, 10)
        for _ in range(warmup):
            _step(m, method)
        ts = [_step(m, method) for _ in range(steps)]
        s = statistics.median([r[0] for r in ts])
        total += s
        per_mesh += [s] * len(g)
        berr_worst = max(berr_worst, ts[-1][1]["berr"])
        iters.append(ts[-1][1]["ir_iters"])
        del m
    out["batched"] = {"s_total": total, "solves_per_s": n_meshes * n_rhs / total,
                      "meshes_per_s": n_meshes / total,
                      "p50_mesh_s": float(np.percentile(per_mesh, 50)),
                      "p99_mesh_s": float(np.percentile(per_mesh, 99)),
                      "worst_backward_error": berr_worst, "max_ir_iters": max(iters)}
    if separate:
        per, berr_worst = [], 0.0
        for s_ in specs:
            m = api.load_spec(s_)
            m.set_mode(1, prec, TOL, 10)
            for _ in range(warmup):
                _step(m, method)
            per.append(statistics.median([_step(m, method)[0] for _ in range(steps)]))
            berr_worst = max(berr_worst, m.timing()["berr"])
            del m
        tot = sum(per)
        out["one_at_a_time"] = {"s_total": tot, "solves_per_s": n_meshes * n_rhs / tot,
                                "meshes_per_s": n_meshes / tot,
                                "p50_mesh_s": float(np.percentile(per, 50)),
                                "p99_mesh_s": float(np.percentile(per, 99)),
                                "worst_backward_error": berr_worst}
        out["batched_speedup"] = tot / total
    return out


def elements(n=16, p=4, seed=0, reps=3):
    t0 = time.perf_counter()
    spec = hpfem.poisson3d(n, p, seed=seed)
    t_host = time.perf_counter() - t0          # the whole host mesh build, element matrices included
    recipe = hpfem.element_recipe(spec)
    m_copy = api.load_spec(spec)
    m_copy.set_mode(1, api.PREC_BF16X3, TOL, 10)
    m_copy.chol_with_free()
    m_copy.solve_chol()
    x_copy = m_copy.node_solution(spec.node_id.astype(np.int32), spec.node_ndof)
    m = api.load_spec(spec, lhs=False)
    m.set_mode(1, api.PREC_BF16X3, TOL, 10)
    m.generate_elements(recipe)
    m.chol_with_free()
    m.solve_chol()
    gen, kern = [], []
    for _ in range(reps):
        t = time.perf_counter()
        m.generate_elements(recipe)            # returns after the kernel has finished
        gen.append(time.perf_counter() - t)
        kern.append(m.timing()["upload_ms"] * 1e-3)   # the generation kernel alone (CUDA events)
    cp = []
    for _ in range(reps):
        t = time.perf_counter()
        m_copy.copy_in_leaves(api.UHM_LHS, spec.mats)   # pageable host buffer -> device element buffer
        cp.append(time.perf_counter() - t)
    m.chol_with_free()
    m.solve_chol()
    x_gen = m.node_solution(spec.node_id.astype(np.int32), spec.node_ndof)
    return {"workload": f"3D Poisson {n}^3 hex p={p} element matrices ({spec.mats.nbytes / 1e6:.0f} MB)",
            "host_mesh_build_s": t_host, "device_generation_s": statistics.median(gen),
            "device_generation_kernel_s": statistics.median(kern),
            "kernel_write_gbs": spec.mats.nbytes / statistics.median(kern) / 1e9,
            "copy_in_s": statistics.median(cp),
            "same_solution_bits": bool(np.array_equal(x_gen, x_copy))}


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m uhm_gb300.measure")
    sub = ap.add_subparsers(dest="what", required=True)
    c = sub.add_parser("convdiff")
    c.add_argument("--n", type=int, default=24)
    c.add_argument("--p", type=int, default=3)
    c.add_argument("--steps", type=int, default=3)
    c.add_argument("--seed", type=int, default=0)
    c.add_argument("--merges", type=int, nargs="*", default=[3, 2, 2, 2])
    c.add_argument("--prec", type=int, default=api.PREC_FP32,
                   help="front precision of the mixed path: 1 FP32, 2 BF16X3 (tensor-core trailing updates)")
    el = sub.add_parser("elements")
    el.add_argument("--n", type=int, default=16)
    el.add_argument("--p", type=int, default=4)
    b = sub.add_parser("batch")
    b.add_argument("--meshes", type=int, default=64)
    b.add_argument("--n-range", type=int, nargs=2, default=(8, 12))
    b.add_argument("--p-range", type=int, nargs=2, default=(2, 4))
    b.add_argument("--rhs", type=int, default=16)
    b.add_argument("--prec", type=int, default=api.PREC_FP32)
    b.add_argument("--max-dofs", type=int, default=6_000_000)
    b.add_argument("--steps", type=int, default=3)
    b.add_argument("--seed", type=int, default=0)
    b.add_argument("--no-separate", action="store_true")
    a = ap.parse_args(argv)
    if a.what == "elements":
        r = elements(a.n, a.p)
    elif a.what == "convdiff":
        r = convdiff(a.n, a.p, a.seed, a.steps, merges=a.merges or None, prec=a.prec)
    elif a.what == "batch":
        r = batch(a.meshes, a.seed, tuple(a.n_range), tuple(a.p_range), a.rhs, a.prec, a.max_dofs,
                  a.steps, separate=not a.no_separate)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
