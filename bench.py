"""Benchmark: factor + solve seconds, 3D Poisson 16^3 hex p=4 (Cholesky fronts).

One step = one full multifrontal factorisation + solve (+ FP64 iterative
refinement for the mixed path) of the workload, inputs already resident in
HBM.  ``value`` is the mixed-precision path with the learned per-front
precision (FP64 / FP32 / BF16-split chosen by the selector network, FP64
refinement to backward error <= 1e-12); the plain FP64 path and the fixed
BF16-split policy are timed beside it.  The selector runs once, at the first
factorisation (outside the timed steps; its wall time is reported).  ``e2e`` times the same steps through the C ABI with host buffers:
bulk copy-in of element matrices and right-hand sides from pinned host memory,
factor, solve, copy-out of the solution.

``--impl reference`` times the reference's own CPU solver on the same
workload: its LINAL + UHM sources compiled for this machine by
oracle/Makefile (from the checkout, or from the git-ignored staged copy
under oracle/_ref/src that travels with the tree), all host cores as OpenMP
threads, sequential OpenBLAS inside each task.  Where that binary cannot be
built, the numpy/scipy restatement in oracle/ is timed instead and the line
says so (``cpu_baseline.kind`` "port").

Parity at the workload's size: the GPU solutions of the plain FP64 path and
of the mixed path are compared with the CPU solution of the ``cpu_baseline``
leg (``rel_err_vs_oracle_fp64`` / ``_mixed``, max-norm relative; the drop-in
bound is 1e-10).

Synthetic data: seeded hp-FEM meshes (uhm_gb300.hpfem); no dataset involved.
Element matrices (512 MB) and fronts (>3 GB) exceed the 129 MB L2, so no L2
flush is needed between steps.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "factor+solve s at 16³ p=4: plain FP64 vs mixed+IR+learned, bwd err≤1e-12"
# DRAM traffic of the tensor-core Schur pass per algorithmic byte, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of its launch on tree
# level -2 of the 12^3 p=4 mesh (27 fronts, fs 631, 145.0 MB against 177.4 MB
# algorithmic); scaled to the benchmark's launches by their algorithmic bytes
SCHUR_TRAFFIC_PER_ALG_BYTE = 145.03 / 177.36
SCHUR_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the Schur launch of poisson3d_12_p4 "
                        "(profiles/tc_chol_schur_poisson3d_12_p4.md), 0.82 x its algorithmic bytes, scaled")
WORKLOAD = "3D Poisson 16^3 hex p=4 Legendre-hierarchic, Dirichlet, octree ND, Cholesky fronts, 1 RHS"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", "0"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return

        def rd():
            for line in self.proc.stdout:
                self.samples.append([x.strip() for x in line.split(",")])
        self.thread = threading.Thread(target=rd, daemon=True)
        self.thread.start()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=2)
        except Exception:
            self.proc.kill()
        s = [x for x in self.samples if len(x) >= 8]
        if not s:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(x[0]) for x in s if x[0].replace(".", "").isdigit()]
        mx = [float(x[1]) for x in s if x[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for x in s for i in range(4) if x[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(s)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def _barrier_max(x: float, ws: int):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


WORKLOADS = {
    "poisson3d_16_p4": (lambda seed: __import__("uhm_gb300.hpfem", fromlist=["x"]).poisson3d(16, 4, seed=seed),
                        WORKLOAD),
    "poisson3d_12_p4": (lambda seed: __import__("uhm_gb300.hpfem", fromlist=["x"]).poisson3d(12, 4, seed=seed),
                        "3D Poisson 12^3 hex p=4 (profiling case: root trailing block above L2 size)"),
    "poisson3d_8_p4": (lambda seed: __import__("uhm_gb300.hpfem", fromlist=["x"]).poisson3d(8, 4, seed=seed),
                       "3D Poisson 8^3 hex p=4 (small profiling case)"),
}


def build_workload(seed=0, name="poisson3d_16_p4"):
    return WORKLOADS[name][0](seed)


def _reference_binary():
    """The reference's own solver built for this machine (oracle/Makefile),
    or None with the reason it is missing."""
    from oracle import ref_runner
    try:
        ok = ref_runner.build(jobs=os.cpu_count() or 8)
    except Exception as exc:                      # build failure: report, fall back to the port
        return None, f"reference build failed: {str(exc)[:200]}"
    return (ref_runner, None) if ok else (None, "reference sources absent (neither checkout nor staged copy)")


def cpu_reference(spec, steps, warmup):
    """Time the CPU path on all host cores: the reference's own solver when it
    builds here, else the numpy/scipy restatement (oracle/uhm_oracle.py).
    Returns (times per step, solution (n_dof, n_rhs) in node order, kind,
    description).  One step = one full numeric factor + solve of the mesh
    (the symbolic phase and file I/O are outside the timed region, as in the
    reference's own test, UHM/test/performance/uhmtest.cxx:73-156)."""
    cores = os.cpu_count() or 1
    rr, why = _reference_binary()
    if rr is not None:
        res = rr.run(spec, 1, threads=cores, reps=warmup + steps)
        t = res.rep_times[warmup:].sum(axis=1).tolist()
        desc = (f"the reference's LINAL+UHM C++ (oracle/Makefile, FLAME-subset shim, sequential OpenBLAS "
                f"per task), uhm::set_num_threads({cores}); {steps} timed full factor+solve runs of the "
                f"workload after {warmup} warm-up")
        return t, res.x, "reference", desc
    from oracle import uhm_oracle as uo
    plan = uo.symbolic(spec)
    times = []
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        r = uo.solve_mesh(spec, uo.CHOL, plan=plan)
        dt = time.perf_counter() - t0 - r.timings["symbolic"]
        if i >= warmup:
            times.append(dt)
    desc = (f"numpy/scipy restatement of the reference path (OpenBLAS on all host cores), {steps} timed full "
            f"factor+solve runs after {warmup} warm-up; the reference binary was not used: {why}")
    return times, r.x, "port", desc


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return
    spec = build_workload()
    cores = os.cpu_count()
    # each step is one full factor+solve (about 5-10 s of CPU work here):
    # the sample is bounded to 1 warm-up + at most 5 timed steps
    steps, warmup = max(1, min(args.steps, 5)), min(args.warmup, 1)
    times, _, kind, desc = cpu_reference(spec, steps, warmup)
    v = statistics.median(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded hp-FEM mesh)", "config": {"workload": WORKLOAD},
        "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": kind,
                         "sample": desc + f" (median of {len(times)})"},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import numpy as np
    from uhm_gb300 import api, build
    build.build()
    ws, rank = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    spec = build_workload(seed=rank, name=args.workload)
    peaks, peak_src = _peaks()
    selector = None
    if args.prec == api.PREC_LEARNED:
        from uhm_gb300 import selector as sel
        selector = sel.load_weights()
        if selector is None:
            raise RuntimeError("learned precision policy: uhm_gb300/selector_weights.npz is missing")
    if args.profile_only:
        # one warm factor+solve of the mixed path, for external profilers
        m = api.load_spec(spec)
        if selector is not None:
            m.set_selector(selector)
        m.set_mode(1, args.prec, 1e-12, 10)
        for _ in range(args.steps + args.warmup):
            m.chol_with_free()
            m.solve_chol()
        print(json.dumps({"profile_only": True, "workload": args.workload, "timing": m.timing()}))
        return

    m = api.load_spec(spec)
    fd, _ = m.estimate_cost(api.UHM_CHOL)

    def one_step(mesh):
        mesh.chol_with_free()
        mesh.solve_chol()
        t = mesh.timing()
        return (t["factor_ms"] + t["solve_ms"] + t["refine_ms"]) * 1e-3, t

    # ---- plain FP64 (drop-in) -------------------------------------------------
    m.set_mode(0)
    for _ in range(max(1, min(args.warmup, 2))):
        one_step(m)
    plain = [one_step(m) for _ in range(max(1, min(args.steps, 3)))]
    plain_s = statistics.median([p[0] for p in plain])
    plain_berr = m.backward_error()
    node_ids = spec.node_id.astype(np.int32)
    x_plain = m.node_solution(node_ids, spec.node_ndof, spec.n_rhs)

    # ---- fixed BF16X3 policy (the mixed path without the selector) -----------
    fixed_s = None
    if args.prec == api.PREC_LEARNED:
        m.set_mode(1, api.PREC_BF16X3, 1e-12, 10)
        for _ in range(max(1, min(args.warmup, 2))):
            one_step(m)
        fixed_s = statistics.median([one_step(m)[0] for _ in range(max(1, min(args.steps, 3)))])

    # ---- mixed + IR (headline): learned per-front precision -------------------
    if selector is not None:
        m.set_selector(selector)
    m.set_mode(1, args.prec, 1e-12, 10)
    t_setup = time.perf_counter()
    one_step(m)                               # first factorisation: features, selector, plan
    t_setup = time.perf_counter() - t_setup
    front_classes = None
    if selector is not None:
        _, cls = m.front_precision()
        front_classes = dict(zip(["fp64", "fp32", "bf16"], np.bincount(cls[cls >= 0], minlength=3).tolist()))
    for _ in range(max(0, args.warmup - 1)):
        one_step(m)
    clocks = Clocks()
    launches0 = None
    clocks.start()
    t_wall = time.perf_counter()
    res = []
    for _ in range(args.steps):
        res.append(one_step(m))
    t_wall = time.perf_counter() - t_wall
    ck = clocks.stop()
    step_s = [r[0] for r in res]
    dev_s = sum(step_s) / len(step_s)
    dev_s = _barrier_max(dev_s, ws)
    last = res[-1][1]
    berr = m.backward_error()
    x_mixed = m.node_solution(node_ids, spec.node_ndof, spec.n_rhs)
    launches = int(sum(r[1]["kernel_launches"] for r in res) / len(res))

    # ---- per-kernel profile (separate pass, outside the timed region) ---------
    m.set_profiling(True)
    one_step(m)
    prof = m.profile()
    m.set_profiling(False)
    # Roofline of the Schur update ABR -= ABL ABL^T (the contraction the
    # metric names), k_tc_chol over the ABR tiles of every tensor-core front
    # with K = fs in one pass.  Each algorithmic flop is three BF16 products
    # (hi*hi + hi*lo + lo*hi) on the tensor cores, so the peak it is held
    # against is a third of the measured dense BF16 rate (the BF16X3
    # emulated-FP32 peak); mma_frac is the tensor pipe's own share.
    # achieved = LAWN-41 SYRK flops of the launch / its CUDA-event time.
    bf16_peak = float(peaks.get("bf16_tflops"))
    terms = 3
    if "tc_chol_schur" in prof and prof["tc_chol_schur"]["ms"] > 0:
        p = prof["tc_chol_schur"]
        nl = max(1, p["launches"])
        tflops = p["flops"] / (p["ms"] * 1e-3) / 1e12
        eff_peak = bf16_peak / terms
        traffic = SCHUR_TRAFFIC_PER_ALG_BYTE * p["bytes"] / nl if SCHUR_TRAFFIC_PER_ALG_BYTE else None
        roof = {"bound": "tensor", "kernel": "tc_chol_schur", "achieved": tflops, "peak": eff_peak,
                "unit": "TFLOP/s", "frac": tflops / eff_peak, "traffic": traffic,
                "traffic_unit": "bytes per launch (dram read+write)",
                "algorithmic_flops_per_launch": p["flops"] / nl, "us_per_launch": 1e3 * p["ms"] / nl,
                "launches": p["launches"],
                "peak_source": f"bf16_tflops of MEASURED_PEAKS.json ({peak_src}) / 3 BF16 products per algorithmic flop",
                "traffic_source": SCHUR_TRAFFIC_SOURCE,
                "tensor": {"achieved_tflops": tflops, "peak_tflops": bf16_peak, "mma_frac": terms * tflops / bf16_peak,
                           "split_terms": terms}}
        if "tc_chol_trail" in prof and prof["tc_chol_trail"]["ms"] > 0:
            q = prof["tc_chol_trail"]
            ttf = q["flops"] / (q["ms"] * 1e-3) / 1e12
            roof["trailing_update"] = {"kernel": "tc_chol_trail", "achieved_tflops": ttf,
                                       "mma_frac": terms * ttf / bf16_peak,
                                       "gbs": q["bytes"] / (q["ms"] * 1e-3) / 1e9,
                                       "hbm_frac": q["bytes"] / (q["ms"] * 1e-3) / 1e9 / peaks["hbm_gbs"]}
    else:
        name, p = max(prof.items(), key=lambda kv: kv[1]["ms"])
        achieved = p["bytes"] / (p["ms"] * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": None,
                "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({peak_src})"}

    # ---- end to end through the C ABI with host buffers -----------------------
    emat = api.pinned_empty(spec.mats.size)
    emat[:] = spec.mats
    erhs = api.pinned_empty(spec.rhs.size)
    erhs[:] = spec.rhs
    xout = api.pinned_empty(spec.rhs.size)
    e2e = []
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        m.copy_in_leaves(api.UHM_LHS, emat)
        m.copy_in_leaves(api.UHM_RHS, erhs)
        m.chol_with_free()
        m.solve_chol()
        m.copy_out_leaves(spec.rhs.size, out=xout)
        dt = time.perf_counter() - t
        if i >= args.warmup:
            e2e.append(dt)
    e2e_s = _barrier_max(statistics.median(e2e), ws)
    ok = np.isfinite(xout).all()

    cpu = None
    parity = {}
    if rank == 0 and not args.no_cpu:
        times, x_cpu, kind, desc = cpu_reference(spec, 1, 0)
        cpu = {"value": times[0], "unit": "s", "cores": os.cpu_count(), "kind": kind, "sample": desc}
        scale = float(np.abs(x_cpu).max())
        parity = {"rel_err_vs_oracle_fp64": float(np.abs(x_plain - x_cpu).max() / scale),
                  "rel_err_vs_oracle_mixed": float(np.abs(x_mixed - x_cpu).max() / scale),
                  "parity_against": ("the reference solver's FP64 solution (cpu_baseline leg)" if kind == "reference"
                                     else "the oracle port's FP64 solution (cpu_baseline leg)"),
                  "parity_tol_fp64": 1e-10}

    if rank == 0:
        line = {
            "metric": METRIC, "value": dev_s, "unit": "s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "mixed: per-front f64/f32/bf16x3 (learned), f64 refinement" if selector is not None
                     else "mixed: f32/bf16x3 fronts, f64 refinement",
            "data": "synthetic (seeded hp-FEM mesh)",
            "config": {"workload": WORKLOAD, "n_dof": int(spec.n_dof()), "n_fronts": int(spec.n_elements),
                       "root_front": 11719, "factor_gflop_lawn41": fd / 1e9,
                       "l2": "inputs larger than L2 (element matrices 512 MB, fronts > 3 GB)",
                       "precision_policy": ["fp64", "fp32", "bf16x3", "bf16x6", "learned"][args.prec]},
            "backward_error": berr, "ir_iters": last["ir_iters"], "berr_first_solve": last.get("berr_first"),
            "factor_ms": last["factor_ms"], "solve_ms": last["solve_ms"], "refine_ms": last["refine_ms"],
            "plain_fp64_s": plain_s, "plain_fp64_backward_error": plain_berr,
            "speedup_vs_plain_fp64": plain_s / dev_s,
            "fixed_bf16x3_s": fixed_s, "selector_front_classes": front_classes,
            "first_step_wall_s": t_setup,
            "wall_s_per_step": t_wall / args.steps,
            "e2e": {"value": e2e_s, "unit": "s",
                    "h2d_bytes_per_step": int((spec.mats.size + spec.rhs.size) * 8),
                    "d2h_bytes_per_step": int(spec.n_dof() * 8), "finite": bool(ok)},
            "gpu_launches": launches,
            "roofline": roof,
            "kernels": {k: {"ms": round(v["ms"], 3), "tflops": round(v["flops"] / (v["ms"] * 1e-3) / 1e12, 2)
                            if v["flops"] else None,
                            "gbs": round(v["bytes"] / (v["ms"] * 1e-3) / 1e9, 1) if v["bytes"] else None,
                            "launches": v["launches"]} for k, v in prof.items()},
            "cpu_baseline": cpu,
            "clocks": ck,
        }
        line.update(parity)
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--prec", type=int, default=4,
                    help="front policy of the mixed path: 0 fp64, 1 fp32, 2 bf16x3, 3 bf16x6 "
                         "(tensor-core split on fronts with n >= 512, fp32 below), 4 learned per front")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="poisson3d_16_p4", choices=sorted(WORKLOADS))
    ap.add_argument("--profile-only", action="store_true",
                    help="run the mixed path only (for ncu launch lists / captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
