#!/usr/bin/env python
"""Benchmark: wall-seconds per converged self-consistent model.

Workload (the rotating NFW configuration): one NFW component with the
double-power-law DF (dphi_h = dz_h = 0.55, dphi_g = dz_g = 1, chi = 1,
k = 0.5, M = r0 = 1), 80 log radii in [1e-3, 300], 40 polar Gauss-Legendre
nodes, even multipoles to l = 12 (npoly = 7), the 22-point-per-axis
tanh-sinh velocity rule (22^3 = 10648 phase-space nodes per grid point) and
20 self-consistency iterations per model.  Inputs are synthetic: the
analytic NFW guess density seeds the first potential (pot/models.cpp:53-56).

A step is one self-consistency iteration over the whole meridional grid
(computeNewPhi: phase-space kernel, Legendre projection, Poisson), chained on
the device as the reference's loop chains them.  value = wall-seconds per
converged model = seconds per step x 20 (whole job: / N for N replicas).

The chosen form is the mixed-precision one (FP32 turning points, momentum
integrals and DF; FP64 node setup, turning points at the u/v limits and
accumulation).  Its density error is measured in the same run: one iteration
from the same input potential in the mixed and the plain FP64 form, max
relative rho difference over all grid points, and the plain form's time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form mixed|plain|gl]
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
           dz_g=1.0, chi=1.0, k=0.5, mass=1.0, r0=1.0, iters_per_model=20, nq=22)
METRIC = "wall-s per converged model at rho err<=1e-4, chosen vs plain FP64, same GB300"
UNIT = "s/model"
# FP64 operations per phase-space evaluation executed by active threads of the
# phase-space kernel (dadd + dmul + 2*dfma from ncu on the nfw_80x40 workload,
# profiles/moments_fp64_nfw_80x40.md); the algorithmic work unit of the roofline.
FP64_FLOPS_PER_EVAL = {"plain": 1.21e5, "gl": None}
# FP32 operations (fadd + fmul + 2*ffma) executed by active lanes per phase-space
# evaluation of the mixed form, from ncu on a 240-point spread of the same workload
# (profiles/moments_mixed_nfw_80x40.md)
FP32_FLOPS_PER_EVAL = {"mixed": 4.68e4}
# DRAM bytes (read + write) per phase-space evaluation from the same captures:
# 1678.2 MB over 2,555,520 evaluations (mixed, the 64-register build with 8 blocks
# per SM; local-memory and partial-sum traffic, the inputs are < 16 KB), 7.58 MB over
# 255,552 (plain FP64); a launch's traffic scales with its evaluations
DRAM_BYTES_PER_EVAL = {"mixed": 1678.2e6 / 2555520, "plain": 7.58e6 / 255552}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="mixed", choices=["mixed", "plain", "gl"])
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison step")
    ap.add_argument("--mixed-config", default=None,
                    help="variant,nodes_per_block of the mixed kernel (default: autotuned before warm-up)")
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="grid points timed for the CPU baseline (default: 10 per host thread for the cpu_baseline "
                         "key, about 10 s; 2 per host thread for each step of --impl reference)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--profile-points", type=int, default=0,
                    help="profiling case: one phase-space launch over this many grid points, no bench line")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4"],
                    help="c2: the bench line (NFW 80x40); c3: a two-component model (64x32, 15 iterations); "
                         "c4: a batched sweep of seeded models (extra measurements, not the bench line)")
    ap.add_argument("--models", type=int, default=256, help="c4: number of models")
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
    if form == "gl":
        return F.Rule(x, w, jquad=16)
    return F.Rule(x, w, precision=A.FJ_PREC_MIXED if form == "mixed" else A.FJ_PREC_FP64)


FORM_TEXT = {"mixed": "mixed precision (FP32 turning points, QAGS momentum integrals and DF; FP64 setup, "
                      "limit turning points and accumulation)",
             "plain": "plain FP64, QAGS momentum integrals",
             "gl": "FP64, 16-point Gauss-Legendre momentum integrals"}
WORKLOAD = (f"NFW rotating (chi=1,k=0.5) {CFG['nr']}x{CFG['ngauss']} grid, l<=12, 22^3 tanh-sinh nodes, "
            f"{CFG['iters_per_model']} iterations/model")


def velocity_rule():
    import fjmodels_gb300 as F
    return F.tanh_sinh_rule(CFG["nq"])


def setup_host():
    """Grid, guess multipoles (host, as the reference does once)."""
    import fjmodels_gb300 as F
    ar = F.log_grid(CFG["rmin"], CFG["rmax"], CFG["nr"])
    rhl = F.guess_rhl(ar, CFG["ngauss"], CFG["npoly"], CFG["model"], CFG["mass"], CFG["r0"])
    return ar, rhl


def run_ours(args, rank, world):
    import torch

    import fjmodels_gb300 as F
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    ctx = F.Context(dev.index)
    nr, ng, npl = CFG["nr"], CFG["ngauss"], CFG["npoly"]
    f64 = dict(dtype=torch.float64, device=dev)
    ar, rhl = setup_host()
    d_ar = torch.tensor(ar, **f64)
    tabs = [torch.zeros((nr, npl), **f64) for _ in range(3)]
    ctx.computePhil(d_ar, torch.tensor(rhl, **f64), *tabs)
    torch.cuda.synchronize()
    E, D, _ = F.tabulate_delta(ar, *[t.cpu().numpy() for t in tabs])
    delta = ctx.delta(torch.tensor(E, **f64), torch.tensor(D, **f64))
    x, w = velocity_rule()
    rule = make_rule(F, args.form, x, w)
    df = F.DFParams(CFG["model"], CFG["dphi_h"], CFG["dz_h"], CFG["dphi_g"], CFG["dz_g"], CFG["chi"], CFG["mass"],
                    CFG["r0"], k=CFG["k"])
    grids = torch.zeros((6, nr, ng), **f64)
    coef = torch.zeros((6, nr, npl), **f64)
    nxt = [torch.zeros((nr, npl), **f64) for _ in range(3)]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2
    tuned = None
    if args.form == "mixed" and args.mixed_config:
        ctx.set_mixed_config(*[int(v) for v in args.mixed_config.split(",")])
        tuned = {"variant": ctx.mixed_config()[0], "nodes_per_block": ctx.mixed_config()[1], "source": "given"}
    elif args.form == "mixed":  # pick the kernel configuration on every 4th grid point (untimed)
        ci, _ = F.gauleg(0, 1, ng)
        allp = np.array([[ar[n] * np.sqrt(1 - c * c), ar[n] * c] for n in range(nr) for c in ci])
        v, c, ms = ctx.autotune_mixed(ctx.potential(d_ar, *tabs), delta, df, rule, torch.tensor(allp[::4], **f64))
        tuned = {"variant": v, "nodes_per_block": c, "sample_kernel_ms": ms, "sample_points": len(allp[::4]),
                 "table_ms": np.round(ctx.autotune_table, 2).tolist(), "table_nodes_per_block": [1024, 2048, 4096]}
    state = {"cur": tabs, "nxt": nxt}
    kernel_ms, changes = [], []

    def step():
        cur, nx = state["cur"], state["nxt"]
        pot = ctx.potential(d_ar, *cur)
        st = ctx.computeNewPhi(pot, delta, df, rule, ng, grids, coef, *nx)
        kernel_ms.append(st.kernel_ms)
        changes.append((nx[0] - cur[0]).abs().div(nx[0][:, :1].abs()).max())
        state["cur"], state["nxt"] = nx, cur
        flush.zero_()
        return st

    for _ in range(args.warmup):
        step()
    kernel_ms.clear()
    torch.cuda.synchronize()
    barrier(world)
    with ClockSampler(dev.index) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        last = None
        for _ in range(args.steps):
            last = step()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
    barrier(world)
    elapsed = max_over_ranks(t1 - t0, world)
    ms_per_step = elapsed / args.steps * 1e3
    value = ms_per_step / 1e3 * CFG["iters_per_model"] / world
    nodes = last.nodes
    k_ms = float(np.mean(kernel_ms))
    fp32 = args.form == "mixed"
    peak = np.zeros(1)
    F.load_library().fj_measure_fma_peak(1 if fp32 else 0, peak.ctypes.data_as(F._abi.DP))
    flops = FP32_FLOPS_PER_EVAL.get(args.form) if fp32 else FP64_FLOPS_PER_EVAL.get(args.form)
    achieved = flops * nodes / (k_ms * 1e-3) / 1e12 if flops else None
    vs_plain = None
    if args.form != "plain" and not args.no_plain:
        vs_plain = compare_plain(F, ctx, d_ar, state["cur"], delta, df, x, w, ng, grids, f64)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if fp32 else "f64",
        "data": "synthetic (analytic NFW guess density, seeded by construction)",
        "config": {"workload": WORKLOAD,
                   "form": FORM_TEXT[args.form],
                   "phase_space_evals_per_step": nodes, "bound_evals_per_step": last.bound,
                   "l2": "256 MiB buffer written between steps", "parallelism": f"replicas{world}"},
        "phase_space_evals_per_s": nodes / (ms_per_step * 1e-3) * world,
        "kernel_ms_per_step": k_ms,
        "potential_change_last": float(changes[-1].item()) if changes else None,
        "gpu_launches": 4 * args.steps,
        "escalated_evals_per_step": last.escalated, "failed_evals_per_step": last.failures,
        "mixed_kernel_config": tuned,
        "vs_plain_fp64": vs_plain,
        "roofline": {"bound": "fp32" if fp32 else "fp64", "kernel": "k_moments_mixed" if fp32 else "k_moments",
                     "achieved": achieved, "peak": float(peak[0]),
                     "unit": "TFLOP/s", "frac": (achieved / peak[0]) if achieved else None,
                     "peak_source": f"fj_measure_fma_peak ({'FP32' if fp32 else 'FP64'} FMA chains, this GPU)",
                     "flops_per_eval": flops,
                     "traffic": (DRAM_BYTES_PER_EVAL[args.form] * nodes) if args.form in DRAM_BYTES_PER_EVAL else None,
                     "traffic_unit": "bytes per launch (ncu capture of a 240-point case, scaled by evaluations)"},
        "clocks": clk.summary(),
    }
    ctx.close()
    return out, (ar, tabs, delta, rule, df)


def compare_plain(F, ctx, d_ar, cur, delta, df, x, w, ng, grids, f64):
    """One iteration from the same potential in the plain FP64 form: its time per model and
    the chosen form's density error against it (max over all grid points of |rho - rho64| /
    rho64; dispersions likewise)."""
    import torch
    pot = ctx.potential(d_ar, *cur)
    nr, npl = cur[0].shape
    coef = torch.zeros((6, nr, npl), **f64)
    outs = [torch.zeros((nr, npl), **f64) for _ in range(3)]
    g64 = torch.zeros_like(grids)
    ctx.computeNewPhi(pot, delta, df, make_rule(F, "mixed", x, w), ng, grids, coef, *outs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = ctx.computeNewPhi(pot, delta, df, make_rule(F, "plain", x, w), ng, g64, coef, *outs)
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    a, b = grids.cpu().numpy().reshape(6, -1), g64.cpu().numpy().reshape(6, -1)
    ok = b[0] > 0
    err = lambda q: float(np.max(np.abs(a[q][ok] - b[q][ok]) / np.abs(b[q][ok])))
    sig_ok = ok & np.isfinite(b[2]) & np.isfinite(b[3]) & np.isfinite(b[4])
    sig = max(float(np.max(np.abs(a[q][sig_ok] - b[q][sig_ok]) / np.abs(b[q][sig_ok]))) for q in (2, 3, 4))
    return {"plain_value": t64 * CFG["iters_per_model"], "unit": UNIT, "plain_kernel_ms": st.kernel_ms,
            "rho_max_rel_err": err(0), "sigma_max_rel_err": sig,
            "note": "one iteration from the same input potential in both forms, all grid points"}


def e2e_ours(args, mixed_cfg=None):
    """Same metric through the host-buffer C-ABI call (fj_run_model): host inputs, device
    compute, host outputs, copies inside the timed region.  One whole model: the one-time
    setup (grid, guess density, Poisson, focal-distance table) and all 20 iterations (each
    with its copy of the new multipoles back to the host for the convergence test), timed
    end to end."""
    import torch

    import fjmodels_gb300 as F
    ctx = F.Context(int(os.environ.get("LOCAL_RANK", "0")))
    if mixed_cfg:
        ctx.set_mixed_config(mixed_cfg["variant"], mixed_cfg["nodes_per_block"])
    x, w = velocity_rule()
    rule = make_rule(F, args.form, x, w)
    df = F.DFParams(CFG["model"], CFG["dphi_h"], CFG["dz_h"], CFG["dphi_g"], CFG["dz_g"], CFG["chi"], CFG["mass"],
                    CFG["r0"], k=CFG["k"])
    its = CFG["iters_per_model"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = ctx.run_model(CFG["nr"], CFG["ngauss"], CFG["npoly"], CFG["rmin"], CFG["rmax"], df, rule, itermax=its)
    wall = time.perf_counter() - t0
    ctx.close()
    setup = r["setup_ms"] * 1e-3
    per_iter = (wall - setup) / its
    nr, ng, npl, ngrid = CFG["nr"], CFG["ngauss"], CFG["npoly"], 30
    h2d = 8 * (nr + nr * npl + 2 * ngrid + 2 * CFG["nq"])
    d2h_step = 8 * nr * npl
    assert r["iterations"] == its
    return {"value": wall, "unit": UNIT, "setup_s": setup, "s_per_iteration": per_iter, "iterations_run": its,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h_step,
            "note": "one fj_run_model call with host buffers, the whole 20-iteration model timed end to end"}


def cpu_sample(args, sample=16):
    """The CPU restatement of the reference (oracle) on a bounded sample of grid points,
    all host threads (one point per thread), extrapolated to a full iteration and a
    20-iteration model."""
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
                chi=CFG["chi"], k=CFG["k"], xq=x, wq=w, jquad=16 if args.form == "gl" else 0)
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
    return {"value": per_iter * CFG["iters_per_model"], "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{sample} of {npts} grid points spread over the grid (22^3 nodes each) on "
                      f"{threads} host threads, one point per thread; extrapolated to {npts} points x "
                      f"{CFG['iters_per_model']} iterations", "sample_s": dt}


def profile_case(args):
    """One phase-space launch over a spread subset of the workload's grid points
    (the small case captured by ncu)."""
    import torch

    import fjmodels_gb300 as F
    ctx = F.Context(0)
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
    df = F.DFParams(CFG["model"], CFG["dphi_h"], CFG["dz_h"], CFG["dphi_g"], CFG["dz_g"], CFG["chi"], CFG["mass"],
                    CFG["r0"], k=CFG["k"])
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
    ctx = F.Context(0)
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
    graph, the focal-distance tables on the GPU), mixed form; 2 iterations timed whole."""
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
    ctx = F.Context(0)
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
        for _ in range(args.warmup):
            cpu_sample(args, sample=4)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            res.append(cpu_sample(args, sample=args.cpu_sample or 2 * os.cpu_count()))
        wall = time.perf_counter() - t0
        v = float(np.mean([r["value"] for r in res]))
        cb = dict(res[-1], value=v)
        print(json.dumps({"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
                          "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic", "config": {"workload": WORKLOAD,
                                                          "form": "the reference's FP64 algorithm on the host "
                                                                  "(the oracle's C restatement)"},
                          "cpu_baseline": cb,
                          "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    out, _ = run_ours(args, rank, world)
    if rank == 0:
        if not args.no_e2e:
            out["e2e"] = e2e_ours(args, out.get("mixed_kernel_config"))
        if not args.no_cpu and world == 1:
            out["cpu_baseline"] = cpu_sample(args, sample=args.cpu_sample or 10 * os.cpu_count())
        print(json.dumps(out))


if __name__ == "__main__":
    main()
