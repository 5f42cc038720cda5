#!/usr/bin/env python
"""Benchmark: wall-seconds per converged self-consistent model.

Workload (the rotating NFW configuration): one NFW component with the
double-power-law DF (dphi_h = dz_h = 0.55, dphi_g = dz_g = 1, chi = 1,
k = 0.5, M = r0 = 1), 80 log radii in [1e-3, 300], 40 polar Gauss-Legendre
nodes, even multipoles to l = 12 (npoly = 7), the 22-point-per-axis
tanh-sinh velocity rule (22^3 = 10648 phase-space nodes per grid point),
iterated from the analytic NFW guess potential until the largest change of a
potential multipole, relative to the monopole of its radius (mergePhi,
include/UtilsLeg.h:266-278), falls below 1e-5.  Inputs are synthetic: the
analytic guess density seeds the first potential (pot/models.cpp:53-56).

A step is one self-consistency iteration over the whole meridional grid
(computeNewPhi: phase-space kernel, Legendre projection, Poisson), chained on
the device as the reference's loop chains them; the timed steps start from
the guess potential.  value = seconds per step x the iterations the model
needs to converge (whole job: / N for N replicas).  e2e = one fj_run_model
call with host buffers that iterates until converged, timed end to end.

The chosen loop mixes each next input potential from the last three outputs
(Anderson, depth 2, mixing factor 1.6: fj_anderson_step) and ends with one
confirming plain step;
the reference iterates the plain map (fJmodels.cpp:131-143), which this
workload needs 19 iterations for.  Against the fixed point (the plain loop
iterated to its 3e-8 floor) the chosen loop's converged density is closer than
the plain loop's.  The plain FP64 comparison and the reference arm keep the
reference's plain loop.

The chosen form is the mixed-precision one (FP32 turning points, momentum
integrals and DF; FP64 node setup, turning points at the u/v limits, FP64
re-solve of any node whose FP32 solve hits a cap, accumulation) with the
cumulative Poisson solve (the radial integrals exact over the interpolated
density, FP64).  With the reference's adaptive Poisson quadrature the loop
does not converge: its answer moves by up to ~1e-3 of the potential between
iterations when a subdivision decision flips.  The plain FP64 form with the
same Poisson solve is measured in the same run: one iteration of each form
from the converged potential gives the chosen form's density error and the
plain form's time per iteration.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form mixed|plain]
  python bench.py --impl reference ...   (the CPU path on this host's cores)
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CFG = dict(model="NFW", nr=80, ngauss=40, npoly=7, rmin=1e-3, rmax=300.0, dphi_h=0.55, dz_h=0.55, dphi_g=1.0,
           dz_g=1.0, chi=1.0, k=0.5, mass=1.0, r0=1.0, nq=22, tol=1e-5, itermax=100, accel=2, accel_beta=1.6)
# iterations the reference's plain loop needs on this workload (measured on the GB300: the
# change falls by ~0.55 per iteration and is 7.8e-6 after the 19th); the reference arm, which
# cannot iterate to convergence in minutes, times one iteration of the reference's algorithm
# and multiplies by it, and so does the plain FP64 comparison
ITERS_PLAIN_LOOP = 19
# iterations of the chosen (mixed) loop (the default number of timed steps)
ITERS_CHOSEN_LOOP = 9
METRIC = "wall-s per converged model at rho err<=1e-4, chosen vs plain FP64, same GB300"
UNIT = "s/model"
# Algorithmic work per phase-space evaluation of this workload: the reference's algorithm
# with every floating-point operation tallied (oracle/count_flops.py on 24 grid points of the
# guess potential): 24,583 add + 29,604 mul + 9,158 div + 897 sqrt + 20 x 3,437 transcendental
# calls = 1.33e5 FLOPs per (grid point, velocity node), bound or not.  The same for both forms
# (the mixed form runs the same algorithm in FP32 with FP64 where FP32 would change decisions).
ALG_FLOPS_PER_EVAL = 1.33e5
# FLOPs executed by active lanes (ncu: fadd + fmul + 2*ffma, resp. the FP64 ones) per
# evaluation in each form's kernel, from captures of the same workload
EXEC_FLOPS_PER_EVAL = {"mixed": 4.68e4, "plain": 1.21e5}
# DRAM bytes (read + write) per phase-space evaluation from ncu captures of the same workload
# (mixed: a 240-point spread, 2,555,520 evaluations; plain: 24 points): local-memory and
# partial-sum traffic, the inputs are < 16 KB; a launch's traffic scales with its evaluations
DRAM_BYTES_PER_EVAL = {"mixed": 1416.7e6 / 2555520, "plain": 7.58e6 / 255552}
L2_NOTE = "256 MiB buffer written between steps"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=ITERS_CHOSEN_LOOP)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="mixed", choices=["mixed", "plain"])
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison step")
    ap.add_argument("--poisson", default="cumulative", choices=["cumulative", "qags"],
                    help="radial Poisson integrals: cumulative (exact over the interpolated density, the chosen "
                         "form) or qags (the reference's adaptive quadrature, which does not let the loop converge)")
    ap.add_argument("--converged-plain", action="store_true",
                    help="also run the plain FP64 form to convergence and compare the converged models (minutes)")
    ap.add_argument("--mixed-config", default=None,
                    help="variant,nodes_per_block of the mixed kernel (default: autotuned before warm-up)")
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="grid points timed for the CPU baseline, spread over the grid (default: 10 per host thread, "
                         "about 6 s on the 16-core box; the same sample for the cpu_baseline key and each step of "
                         "--impl reference)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the two-component (c3) and batched-sweep (c4) measurements added to the line")
    ap.add_argument("--profile-points", type=int, default=0,
                    help="profiling case: one phase-space launch over this many grid points, no bench line")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4"],
                    help="c2: the bench line (NFW 80x40); c3: a two-component model (64x32, 15 iterations); "
                         "c4: a batched sweep of seeded models (extra measurements, not the bench line)")
    ap.add_argument("--models", type=int, default=256, help="c4: number of models")
    ap.add_argument("--loop-study", action="store_true",
                    help="the workload's loop to convergence in the mixed form: the plain loop and Anderson-mixed "
                         "loops (depths 1, 2, 3, 5; mixing factors 1, 1.3, 1.6, 2 at depth 2) against the fixed point "
                         "(the plain loop run 42 times); no bench line")
    return ap.parse_args()


def dist_init():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
    return rank, world


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                try:
                    rows.append((float(parts[1]), float(parts[2]), parts[4:8]))
                except ValueError:
                    pass
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for _, _, r in rows for n, v in zip(names, r) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def make_rule(F, form, x, w):
    from fjmodels_gb300 import _abi as A
    return F.Rule(x, w, precision=A.FJ_PREC_MIXED if form == "mixed" else A.FJ_PREC_FP64)


FORM_TEXT = {"mixed": "mixed precision (FP32 turning points, QAGS momentum integrals and DF; FP64 setup, "
                      "limit turning points, re-solve of capped nodes and accumulation), cumulative Poisson solve",
             "plain": "plain FP64, QAGS momentum integrals, cumulative Poisson solve"}
WORKLOAD = (f"NFW rotating (chi=1,k=0.5) {CFG['nr']}x{CFG['ngauss']} grid, l<=12, 22^3 tanh-sinh nodes, "
            f"iterated to max|dphil/phil_0| < {CFG['tol']:g}")


def velocity_rule():
    import fjmodels_gb300 as F
    return F.tanh_sinh_rule(CFG["nq"])


def setup_host():
    """Grid, guess multipoles (host, as the reference does once)."""
    import fjmodels_gb300 as F
    ar = F.log_grid(CFG["rmin"], CFG["rmax"], CFG["nr"])
    rhl = F.guess_rhl(ar, CFG["ngauss"], CFG["npoly"], CFG["model"], CFG["mass"], CFG["r0"])
    return ar, rhl


def df_params(F):
    return F.DFParams(CFG["model"], CFG["dphi_h"], CFG["dz_h"], CFG["dphi_g"], CFG["dz_g"], CFG["chi"], CFG["mass"],
                      CFG["r0"], k=CFG["k"])


POISSON = {"mode": "cumulative"}


def new_context(F, index):
    from fjmodels_gb300 import _abi as A
    ctx = F.Context(index)
    ctx.set_poisson(A.FJ_POISSON_CUMULATIVE if POISSON["mode"] == "cumulative" else A.FJ_POISSON_QAGS)
    return ctx


def run_ours(args, rank, world):
    import torch

    import fjmodels_gb300 as F
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    ctx = new_context(F, dev.index)
    nr, ng, npl = CFG["nr"], CFG["ngauss"], CFG["npoly"]
    f64 = dict(dtype=torch.float64, device=dev)
    ar, rhl = setup_host()
    d_ar = torch.tensor(ar, **f64)
    guess = [torch.zeros((nr, npl), **f64) for _ in range(3)]
    ctx.computePhil(d_ar, torch.tensor(rhl, **f64), *guess)
    torch.cuda.synchronize()
    E, D, _ = F.tabulate_delta(ar, *[t.cpu().numpy() for t in guess])
    delta = ctx.delta(torch.tensor(E, **f64), torch.tensor(D, **f64))
    x, w = velocity_rule()
    rule = make_rule(F, args.form, x, w)
    df = df_params(F)
    grids = torch.zeros((6, nr, ng), **f64)
    coef = torch.zeros((6, nr, npl), **f64)
    bufs = [torch.zeros((3, nr, npl), **f64) for _ in range(2)]  # phil, Pr, Pr2 of the input and the output
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2
    tuned = None
    if args.form == "mixed" and args.mixed_config:
        ctx.set_mixed_config(*[int(v) for v in args.mixed_config.split(",")])
        tuned = {"variant": ctx.mixed_config()[0], "nodes_per_block": ctx.mixed_config()[1], "source": "given"}
    elif args.form == "mixed":  # pick the kernel configuration on every 4th grid point (untimed)
        ci, _ = F.gauleg(0, 1, ng)
        allp = np.array([[ar[n] * np.sqrt(1 - c * c), ar[n] * c] for n in range(nr) for c in ci])
        pot0 = ctx.potential(d_ar, *guess)
        v, c, ms = ctx.autotune_mixed(pot0, delta, df, rule, torch.tensor(allp[::4], **f64))
        tuned = {"variant": v, "nodes_per_block": c, "sample_kernel_ms": ms, "sample_points": len(allp[::4]),
                 "table_ms": np.round(ctx.autotune_table, 2).tolist(), "table_nodes_per_block": [1024, 2048, 4096]}
        # The sample can rank the builds within its noise (~1 %) while they differ by up to
        # ~20 % on the whole grid (the block count sets the load balance there): the three
        # fastest on the sample are timed again on every grid point of the guess potential
        # (the better of two launches each) and the fastest there is kept.
        chunks = tuned["table_nodes_per_block"]
        cands = sorted((t, vv, chunks[cc]) for vv, row in enumerate(ctx.autotune_table) for cc, t in enumerate(row))[:3]
        pts, out6 = torch.tensor(allp, **f64), torch.zeros((6, len(allp)), **f64)
        confirm = {}
        for _, vv, cc in cands:
            ctx.set_mixed_config(int(vv), int(cc))
            confirm[f"{vv},{cc}"] = round(min(ctx.moments_points(pot0, delta, df, rule, pts, out6).kernel_ms
                                              for _ in range(2)), 2)
        best = min(confirm, key=confirm.get)
        ctx.set_mixed_config(*[int(t) for t in best.split(",")])
        tuned.update(variant=ctx.mixed_config()[0], nodes_per_block=ctx.mixed_config()[1], full_grid_ms=confirm)
    state = {}

    accel = CFG["accel"] if args.form == "mixed" else 0

    def restart():  # the model's first iteration starts from the guess potential
        for b, g in zip(bufs[0], guess):
            b.copy_(g)
        state.update(cur=bufs[0], nxt=bufs[1], confirmed=False, converged_at=None)
        if accel:
            ctx.anderson_reset(accel, CFG["accel_beta"])

    kernel_ms, changes, stats = [], [], []

    def step():
        # one iteration of fj_run_model's loop: computeNewPhi, the change, then a plain step
        # (the output is the next input) or, in the chosen loop, a mixed one (fj_anderson_step)
        cur, nx = state["cur"], state["nxt"]
        pot = ctx.potential(d_ar, *cur)
        st = ctx.computeNewPhi(pot, delta, df, rule, ng, grids, coef, *nx)
        kernel_ms.append(st.kernel_ms)
        stats.append(st)
        change = float((nx[0] - cur[0]).abs().div(nx[0][:, :1].abs()).max())
        changes.append(change)
        below = change < CFG["tol"]
        if not accel or below:
            state["cur"], state["nxt"] = nx, cur
            if below and (not accel or state["confirmed"]) and state["converged_at"] is None:
                state["converged_at"] = len(changes)
            state["confirmed"] = below
        else:
            ctx.anderson_step(cur, nx)
            state["confirmed"] = False
        flush.zero_()
        return st

    restart()
    for _ in range(args.warmup):
        step()
    restart()
    kernel_ms.clear()
    changes.clear()
    stats.clear()
    torch.cuda.synchronize()
    barrier(world)
    with ClockSampler(dev.index) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
    barrier(world)
    elapsed = max_over_ranks(t1 - t0, world)
    ms_per_step = elapsed / args.steps * 1e3
    ch = list(changes)
    conv_timed = state["converged_at"]
    nodes = stats[-1].nodes
    k_ms = float(np.mean(kernel_ms))
    fp32 = args.form == "mixed"
    peak = np.zeros(1)
    F.load_library().fj_measure_fma_peak(1 if fp32 else 0, peak.ctypes.data_as(F._abi.DP))
    achieved = ALG_FLOPS_PER_EVAL * nodes / (k_ms * 1e-3) / 1e12
    executed = EXEC_FLOPS_PER_EVAL[args.form] * nodes / (k_ms * 1e-3) / 1e12
    tot = lambda f: int(sum(getattr(st, f) for st in stats))  # noqa: E731
    out = {
        "metric": METRIC, "value": None, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if fp32 else "f64",
        "data": "synthetic (analytic NFW guess density, seeded by construction)",
        "config": {"workload": WORKLOAD, "l2": L2_NOTE},
        "form": FORM_TEXT[args.form] + ("" if args.poisson == "cumulative" else " (adaptive QAGS Poisson solve)"),
        "parallelism": f"replicas{world}",
        "phase_space_evals_per_step": nodes, "bound_evals_per_step": stats[-1].bound,
        "phase_space_evals_per_s": nodes / (ms_per_step * 1e-3) * world,
        "kernel_ms_per_step": k_ms,
        "tol": CFG["tol"], "potential_change_per_timed_step": [float(f"{c:.3g}") for c in ch],
        "iterations_to_converge_timed": conv_timed,
        "gpu_launches": 4 * args.steps,
        "failed_evals_timed": tot("failures"), "failed_by_kind_timed": {"quad": tot("fail_quad"),
                                                                        "bracket": tot("fail_bracket"),
                                                                        "root": tot("fail_root")},
        "resolved_fp64_evals_per_step": tot("resolved64") / len(stats), "escalated_evals_timed": tot("escalated"),
        "mixed_kernel_config": tuned,
        "roofline": {"bound": "fp32" if fp32 else "fp64", "kernel": "k_moments_mixed" if fp32 else "k_moments",
                     "achieved": achieved, "peak": float(peak[0]),
                     "unit": "TFLOP/s", "frac": achieved / peak[0],
                     "peak_source": f"fj_measure_fma_peak ({'FP32' if fp32 else 'FP64'} FMA chains, this GPU; "
                                    "the measured peaks file covers HBM and BF16 only)",
                     "flops_per_eval": ALG_FLOPS_PER_EVAL,
                     "flops_source": "algorithmic: the reference's algorithm with its operations tallied "
                                     "(oracle/count_flops.py), transcendental calls weighted 20",
                     "executed_achieved": executed, "executed_frac": executed / peak[0],
                     "executed_flops_per_eval": EXEC_FLOPS_PER_EVAL[args.form],
                     "traffic": (DRAM_BYTES_PER_EVAL[args.form] * nodes) if args.form in DRAM_BYTES_PER_EVAL else None,
                     "traffic_unit": "bytes per launch (ncu capture of a 240-point case, scaled by evaluations)"},
        "clocks": clk.summary(),
    }
    ctx.close()
    return out, dict(d_ar=d_ar, delta=delta, rule=rule, df=df, x=x, w=w, f64=f64)


def plain_at(F, env, tabs_host, iters):
    """One iteration of each form from the same (converged) potential: the plain FP64 form's
    time per iteration and the chosen form's density error against it (max over all grid
    points of |rho - rho64| / rho64; the second moments likewise; the density multipoles
    relative to the monopole of their radius)."""
    import torch
    ctx = new_context(F, torch.cuda.current_device())
    f64, d_ar, delta, df = env["f64"], env["d_ar"], env["delta"], env["df"]
    nr, npl = tabs_host[0].shape
    ng = CFG["ngauss"]
    cur = [torch.tensor(np.ascontiguousarray(t), **f64) for t in tabs_host]
    pot = ctx.potential(d_ar, *cur)
    outs = [torch.zeros((nr, npl), **f64) for _ in range(3)]
    res = {}
    for form in ("mixed", "plain"):
        g = torch.zeros((6, nr, ng), **f64)
        c = torch.zeros((6, nr, npl), **f64)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = ctx.computeNewPhi(pot, delta, df, make_rule(F, form, env["x"], env["w"]), ng, g, c, *outs)
        torch.cuda.synchronize()
        res[form] = (g.cpu().numpy().reshape(6, -1), c.cpu().numpy(), time.perf_counter() - t0, st)
    ctx.close()
    a, b = res["mixed"][0], res["plain"][0]
    ok = b[0] > 0
    err = float(np.max(np.abs(a[0][ok] - b[0][ok]) / np.abs(b[0][ok])))
    sig_ok = ok & np.isfinite(b[2]) & np.isfinite(b[3]) & np.isfinite(b[4])
    sig = max(float(np.max(np.abs(a[q][sig_ok] - b[q][sig_ok]) / np.abs(b[q][sig_ok]))) for q in (2, 3, 4))
    ca, cb = res["mixed"][1][0], res["plain"][1][0]
    rhl_err = float(np.max(np.abs(ca - cb) / np.abs(cb[:, :1])))
    t64 = res["plain"][2]
    return {"plain_s_per_iteration": t64, "plain_value": t64 * ITERS_PLAIN_LOOP, "unit": UNIT,
            "plain_value_chosen_loop": t64 * iters,
            "plain_kernel_ms": res["plain"][3].kernel_ms, "plain_failures": res["plain"][3].failures,
            "rho_max_rel_err": err, "sigma_max_rel_err": sig, "rhl_max_rel_err": rhl_err,
            "note": f"one iteration of each form from the chosen form's converged potential, all grid points; "
                    f"plain_value = its time x the {ITERS_PLAIN_LOOP} iterations of the reference's plain loop "
                    f"(plain_value_chosen_loop: x the chosen loop's {iters})"}


def run_model_host(F, ctx, form, itermax, accel=0, tol=None, beta=None):
    x, w = velocity_rule()
    return ctx.run_model(CFG["nr"], CFG["ngauss"], CFG["npoly"], CFG["rmin"], CFG["rmax"], df_params(F),
                         make_rule(F, form, x, w), itermax=itermax, tol=CFG["tol"] if tol is None else tol, accel=accel,
                         accel_beta=CFG["accel_beta"] if beta is None else beta)


def loop_study(args):
    """Iterations and distance to the fixed point of each loop (mixed form): the potential
    (max |dphil| / |phil(r, 0)|) and the density multipoles (relative to each shell's
    monopole, with the shell of the largest difference)."""
    import fjmodels_gb300 as F
    ctx = new_context(F, 0)
    ctx.set_mixed_config(*[int(v) for v in (args.mixed_config or "7,1024").split(",")])
    fixed = run_model_host(F, ctx, "mixed", 42, tol=0.0)
    rows = {"fixed_point": {"iterations": fixed["iterations"], "last_change": fixed["last_change"]}}
    s0, rho0 = np.abs(fixed["phil"][:, :1]), fixed["coef6"][0]
    for m, beta in ((0, 1.0), (1, 1.0), (2, 1.0), (3, 1.0), (5, 1.0), (2, 1.3), (2, 1.6), (2, 2.0)):
        r = run_model_host(F, ctx, "mixed", CFG["itermax"], accel=m, beta=beta)
        e = np.abs(r["coef6"][0] - rho0) / np.abs(rho0[:, :1])
        rows["plain" if m == 0 else f"anderson{m}_beta{beta:g}"] = {
            "iterations": r["iterations"], "last_change": r["last_change"],
            "potential": float(np.max(np.abs(r["phil"] - fixed["phil"]) / s0)),
            "density_multipoles": float(np.max(e)), "worst_shell": int(np.unravel_index(np.argmax(e), e.shape)[0])}
    ctx.close()
    print(json.dumps({"loop_study": rows, "workload": WORKLOAD, "tol": CFG["tol"]}))


def e2e_ours(args, mixed_cfg=None):
    """Same metric through the host-buffer C-ABI call (fj_run_model): host inputs, device
    compute, host outputs, copies inside the timed region.  One whole model: the one-time
    setup (grid, guess density, Poisson, focal-distance table) and every iteration until the
    model has converged (each with its copy of the new multipoles back to the host for the
    convergence test), timed end to end."""
    import torch

    import fjmodels_gb300 as F
    ctx = new_context(F, int(os.environ.get("LOCAL_RANK", "0")))
    if mixed_cfg:
        ctx.set_mixed_config(mixed_cfg["variant"], mixed_cfg["nodes_per_block"])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = run_model_host(F, ctx, args.form, CFG["itermax"], CFG["accel"] if args.form == "mixed" else 0)
    wall = time.perf_counter() - t0
    ctx.close()
    setup = r["setup_ms"] * 1e-3
    its = r["iterations"]
    nr, ng, npl, ngrid = CFG["nr"], CFG["ngauss"], CFG["npoly"], 30
    h2d = 8 * (nr + nr * npl + 2 * ngrid + 2 * CFG["nq"])
    d2h_step = 8 * nr * npl
    converged = r["last_change"] < CFG["tol"]
    return {"value": wall, "unit": UNIT, "setup_s": setup, "s_per_iteration": (wall - setup) / its,
            "iterations_to_converge": its if converged else None, "converged": converged,
            "last_change": r["last_change"], "failures": r["failures"],
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h_step,
            "note": "one fj_run_model call with host buffers, iterated until converged, timed end to end"}, r


def converged_plain(F, r_mixed):
    """The plain FP64 form run to convergence the same way; the two converged models'
    density multipoles compared (relative to the monopole of their radius)."""
    import torch
    ctx = new_context(F, torch.cuda.current_device())
    t0 = time.perf_counter()
    r = run_model_host(F, ctx, "plain", CFG["itermax"])
    wall = time.perf_counter() - t0
    ctx.close()
    a, b = r_mixed["coef6"][0], r["coef6"][0]
    return {"plain_value": wall, "plain_iterations": r["iterations"], "plain_last_change": r["last_change"],
            "plain_failures": r["failures"], "rhl_max_rel_err": float(np.max(np.abs(a - b) / np.abs(b[:, :1]))),
            "phil_max_rel_err": float(np.max(np.abs(r_mixed["phil"] - r["phil"]) / np.abs(r["phil"][:, :1]))),
            "note": "both forms iterated to convergence through fj_run_model, converged multipoles compared"}


def cpu_sample(args, sample=16):
    """The CPU restatement of the reference (oracle) on a bounded sample of grid points,
    all host threads (one point per thread), extrapolated to a full iteration and to the
    iterations a converged model needs."""
    import ctypes as C
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    nr, ng, npl = CFG["nr"], CFG["ngauss"], CFG["npoly"]
    ar = O.log_grid(CFG["rmin"], CFG["rmax"], nr)
    rhl = O.guess_rhl(ar, ng, npl, CFG["model"], CFG["mass"], CFG["r0"])
    phil, Pr, Pr2 = O.compute_phil(ar, rhl)
    x, w = velocity_rule()
    m = O.Model(ar, phil, Pr, Pr2, np.zeros(30), np.zeros(30), ng, alpha=1.667, beta=3.0, mass=CFG["mass"],
                r0=CFG["r0"], dphi_h=CFG["dphi_h"], dz_h=CFG["dz_h"], dphi_g=CFG["dphi_g"], dz_g=CFG["dz_g"],
                chi=CFG["chi"], k=CFG["k"], xq=x, wq=w)
    E, D, _ = m.tabulate_delta(30)
    m.Egrid, m.Dgrid = E, D
    npts = nr * ng
    idx = np.linspace(0, npts - 1, sample).astype(int)
    threads = os.cpu_count()
    out = np.zeros((6, npts))
    mc = m.c()
    lib = O.lib()

    def one(p):  # ctypes drops the GIL for the call
        lib.orc_moment_grid(mc, int(p), int(p) + 1, out.ctypes.data_as(O.DP), 1, C.byref(O.Stats()))

    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(one, idx))
    dt = time.perf_counter() - t0
    per_iter = dt * npts / sample  # sample points took dt on the host's threads
    return {"value": per_iter * ITERS_PLAIN_LOOP, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{sample} of {npts} grid points spread over the grid (22^3 nodes each) on "
                      f"{threads} host threads, one point per thread; extrapolated to {npts} points x "
                      f"{ITERS_PLAIN_LOOP} iterations", "sample_s": dt}


def profile_case(args):
    """One phase-space launch over a spread subset of the workload's grid points
    (the small case captured by ncu)."""
    import torch

    import fjmodels_gb300 as F
    ctx = new_context(F, 0)
    nr, ng, npl = CFG["nr"], CFG["ngauss"], CFG["npoly"]
    f64 = dict(dtype=torch.float64, device="cuda")
    ar, rhl = setup_host()
    d_ar = torch.tensor(ar, **f64)
    tabs = [torch.zeros((nr, npl), **f64) for _ in range(3)]
    ctx.computePhil(d_ar, torch.tensor(rhl, **f64), *tabs)
    torch.cuda.synchronize()
    E, D, _ = F.tabulate_delta(ar, *[t.cpu().numpy() for t in tabs])
    delta = ctx.delta(torch.tensor(E, **f64), torch.tensor(D, **f64))
    x, w = velocity_rule()
    rule = make_rule(F, args.form, x, w)
    df = df_params(F)
    ci, _ = F.gauleg(0, 1, ng)
    allp = np.array([[ar[n] * np.sqrt(1 - c * c), ar[n] * c] for n in range(nr) for c in ci])
    pts = torch.tensor(allp[np.linspace(0, nr * ng - 1, args.profile_points).astype(int)], **f64)
    out = torch.zeros((6, pts.shape[0]), **f64)
    if args.form == "mixed" and args.mixed_config:
        ctx.set_mixed_config(*[int(v) for v in args.mixed_config.split(",")])
    st = ctx.moments_points(ctx.potential(d_ar, *tabs), delta, df, rule, pts, out)
    torch.cuda.synchronize()
    print(json.dumps({"profile_points": pts.shape[0], "nodes": st.nodes, "bound": st.bound,
                      "kernel_ms": st.kernel_ms, "failures": st.failures}))


def workload_c3(args):
    """Two-component model: Hernquist bulge (M = 0.1, r0 = 1) + NFW halo (M = 1, r0 = 10), each
    component's h/g coefficients drawn from U[0.4, 1.0] with a fixed seed; 64 x 32 grid, l <= 10,
    22^3 tanh-sinh nodes, the summed density in one Poisson solve, 15 iterations, mixed form."""
    import fjmodels_gb300 as F
    from fjmodels_gb300 import _abi as A
    rng = np.random.default_rng(2024)
    d1, d2 = rng.uniform(0.4, 1.0, 4), rng.uniform(0.4, 1.0, 4)
    bulge = F.DFParams("Hernquist", *d1, mass=0.1, r0=1.0)
    halo = F.DFParams("NFW", *d2, mass=1.0, r0=10.0)
    ctx = new_context(F, 0)
    rule = F.Rule(*velocity_rule(), precision=A.FJ_PREC_MIXED)
    nr, ng, npl, it = 64, 32, 6, 15
    out = ctx.run_model(nr, ng, npl, 1e-3, 300.0, bulge, rule, itermax=it, df2=halo,
                        twocomp_order=A.FJ_TWOCOMP_SUMMED)
    evals = 2 * nr * ng * CFG["nq"] ** 3 * it
    ctx.close()
    return {"workload": "c3", "metric": "wall-s per two-component model (64x32, l<=10, 15 iterations, mixed form)",
            "value": out["wall_ms"] / 1e3, "unit": "s/model", "setup_s": out["setup_ms"] / 1e3,
            "kernel_s": out["kernel_ms"] / 1e3, "phase_space_evals_per_s": evals / (out["wall_ms"] / 1e3),
            "iterations": out["iterations"], "dfs": {"bulge": d1.round(4).tolist(), "halo": d2.round(4).tolist()},
            "data": "synthetic (seeded DF draw, analytic guess densities)"}


def workload_c4(args):
    """Batched sweep: seeded models -- type from {Hernquist, Isochrone, NFW}, h/g coefficients
    ~ U[0.3, 1.2], chi ~ U[0, 2], radii in {32, 48, 64, 96} x angles in {16, 24, 32}, l <= 8 --
    iterated together (one phase-space launch per iteration, the iteration captured as a CUDA
    graph, the focal-distance tables on the GPU), mixed form; 2 iterations timed whole.  The
    phase-space launch is one persistent kernel that takes (model, point, node range) items
    from a work queue, most expensive first."""
    import fjmodels_gb300 as F
    from fjmodels_gb300 import _abi as A
    rng = np.random.default_rng(256)
    models = []
    for _ in range(args.models):
        kind = ["Hernquist", "Isochrone", "NFW"][rng.integers(3)]
        dh = rng.uniform(0.3, 1.2, 4)
        df = F.DFParams(kind, *dh, chi=float(rng.uniform(0, 2)), k=0.5)
        models.append(dict(nr=int(rng.choice([32, 48, 64, 96])), ngauss=int(rng.choice([16, 24, 32])), npoly=5,
                           rmin=1e-3, rmax=300.0 if kind == "NFW" else 100.0, df=df))
    ctx = new_context(F, 0)
    rule = F.Rule(*velocity_rule(), precision=A.FJ_PREC_MIXED)
    it = 2
    outs = ctx.run_model_batch(models, rule, itermax=it, use_graph=True, delta_gpu=True)
    o = outs[0]
    evals = sum(m["nr"] * m["ngauss"] for m in models) * CFG["nq"] ** 3 * it
    ctx.close()
    return {"workload": "c4", "metric": f"wall-s per batched iteration of {len(models)} models (mixed form)",
            "value": (o["wall_ms"] - o["setup_ms"]) / 1e3 / it, "unit": "s/iteration", "setup_s": o["setup_ms"] / 1e3,
            "models": len(models), "grid_points": sum(m["nr"] * m["ngauss"] for m in models),
            "phase_space_evals_per_s": evals / ((o["wall_ms"] - o["setup_ms"]) / 1e3),
            "data": "synthetic (seeded model draw, analytic guess densities)"}


def main():
    args = parse()
    POISSON["mode"] = args.poisson
    if args.loop_study:
        return loop_study(args)
    if args.profile_points:
        profile_case(args)
        return
    if args.workload != "c2":
        print(json.dumps(workload_c3(args) if args.workload == "c3" else workload_c4(args)))
        return
    rank, world = dist_init()
    if args.impl == "reference":
        if rank != 0:
            return
        res = []
        flush = np.empty(256 * 1024 * 1024 // 8)  # host caches flushed between steps
        for _ in range(args.warmup):
            cpu_sample(args, sample=4)
            flush.fill(0.0)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            res.append(cpu_sample(args, sample=args.cpu_sample or 10 * os.cpu_count()))
            flush.fill(0.0)
        wall = time.perf_counter() - t0
        v = float(np.mean([r["value"] for r in res]))
        cb = dict(res[-1], value=v)
        print(json.dumps({"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
                          "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic (analytic NFW guess density, seeded by construction)",
                          "config": {"workload": WORKLOAD, "l2": L2_NOTE},
                          "form": "the reference's FP64 algorithm on the host (the oracle's C restatement): one "
                                  f"iteration, sampled, x {ITERS_PLAIN_LOOP} iterations",
                          "cpu_baseline": cb,
                          "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    out, env = run_ours(args, rank, world)
    import fjmodels_gb300 as F
    e2e, r = (None, None) if args.no_e2e else e2e_ours(args, out.get("mixed_kernel_config"))
    iters = (e2e or {}).get("iterations_to_converge") or out["iterations_to_converge_timed"]
    out["iterations_to_converge"] = iters
    out["value"] = out["ms_per_step"] * 1e-3 * iters / world if iters else None
    if rank == 0:
        if e2e:
            out["e2e"] = e2e
        if args.form == "mixed" and not args.no_plain and r is not None:
            out["vs_plain_fp64"] = plain_at(F, env, (r["phil"], r["Pr"], r["Pr2"]), iters or ITERS_PLAIN_LOOP)
            if args.converged_plain:
                out["vs_plain_fp64"]["converged"] = converged_plain(F, r)
        if not args.no_cpu and world == 1:
            out["cpu_baseline"] = cpu_sample(args, sample=args.cpu_sample or 10 * os.cpu_count())
        if not args.no_extra and world == 1 and args.form == "mixed":
            out["extra_workloads"] = {"c3": workload_c3(args), "c4": workload_c4(args)}
        print(json.dumps(out))


if __name__ == "__main__":
    main()
