"""Host-side mirror of the reference's interfaces over the C ABI.

Names follow the reference: ``rhofDF`` grids (integ/Integ.cpp), ``computeNewPhi``
(pot/potLeg.cpp), ``computePhil`` (pot/Potential.cpp), ``uvOrb`` actions
(uvOrb/uvOrb.cpp), ``vir2`` (libs/Stats.cpp), ``writeOut`` (io/writeOut.cpp),
``readParam`` (io/readParam.cpp).  Device arrays are torch CUDA tensors
(float64, contiguous); torch only provides the memory and the stream.  There is
no CPU fallback: every compute call goes to libfjgpu.so and raises if the
library or the GPU is unavailable.
"""
import ctypes as C
import os

import numpy as np

from . import _abi as A

# the reference's live velocity rule, include/GaussPts.h:79-88 (QUAD22 "rectangle method")
XPT11 = np.array([-1., -0.50118723, -0.25118864, -0.12589254, -0.06309573,
                  -0.03162278, -0.01584893, -0.00794328, -0.00398107, -0.00199526,
                  -0.001, 0.001, 0.00199526, 0.00398107, 0.00794328,
                  0.01584893, 0.03162278, 0.06309573, 0.12589254, 0.25118864,
                  0.50118723, 1.])
XW11 = np.array([0.49881277, 0.37440568, 0.18764735, 0.09404645, 0.04713488,
                 0.0236234, 0.01183975, 0.00593393, 0.00297401, 0.00149054,
                 0.00149763, 0.00149763, 0.00149054, 0.00297401, 0.00593393,
                 0.01183975, 0.0236234, 0.04713488, 0.09404645, 0.18764735,
                 0.37440568, 0.49881277])

# DF slopes selected by model name (df/DF.cpp:40-43)
MODEL_SLOPES = {"Hernquist": (1.667, 5.0), "Isochrone": (0.0, 5.0), "NFW": (1.667, 3.0)}


class FJError(RuntimeError):
    pass


def _dp(a):
    return a.ctypes.data_as(A.DP)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(t):
    """Device pointer of a torch CUDA float64 tensor (or an int address)."""
    if isinstance(t, int):
        return t
    if not t.is_cuda or not t.is_contiguous():
        raise FJError("device arrays must be contiguous CUDA tensors")
    return t.data_ptr()


def tanh_sinh_rule(n=22, eps=1e-5):
    """n-point composite tanh-sinh (double-exponential) rule on [-1,1]
    (Takahasi & Mori 1974): n/2 nodes of the rule on [0,1],
    x_k = (1 + tanh(pi/2 sinh(k h)))/2, w_k = h pi/4 cosh(k h) / cosh^2(pi/2 sinh(k h)),
    k = -(m-1)/2 .. (m-1)/2, mirrored onto [-1,0].  Nodes cluster at v = 0 and at
    |v| = 1 like the reference's [0,1] tanh-sinh table (include/GaussPts.h:91-134);
    h puts the outermost node at distance eps from the ends.  Each half's weights
    are normalised to 1."""
    if n % 2:
        raise ValueError("n must be even")
    m = n // 2
    ks = np.arange(m) - (m - 1) / 2.0
    kmax = ks[-1]
    h = np.arcsinh(np.arctanh(1 - 2 * eps) * 2 / np.pi) / kmax
    u = np.pi / 2 * np.sinh(ks * h)
    x = 0.5 * (1 + np.tanh(u))
    w = h * np.pi / 4 * np.cosh(ks * h) / np.cosh(u) ** 2
    w = w / w.sum()
    return np.concatenate([-x[::-1], x]), np.concatenate([w[::-1], w])


class DFParams:
    """DF of one component (df/DF.cpp:36-63): slopes from the model name, J0 = sqrt(M r0)."""

    def __init__(self, model="Hernquist", dphi_h=0.55, dz_h=0.55, dphi_g=1.0, dz_g=1.0, chi=0.0, mass=1.0,
                 r0=1.0, k=0.5, kind=A.FJ_DF_DPL, alpha=None, beta=None):
        a, b = MODEL_SLOPES.get(model, (alpha, beta))
        if alpha is not None and model not in MODEL_SLOPES:
            a, b = alpha, beta
        if a is None or b is None:
            raise FJError("either set a known model or alpha and beta")
        self.c = A.fj_df_params(kind, a, b, float(np.sqrt(mass * r0)), mass, dphi_h, dz_h, dphi_g, dz_g, chi, k)
        self.model, self.mass, self.r0 = model, mass, r0


class Rule:
    """Velocity rule (same on the three axes) + momentum-integral rule + arithmetic."""

    def __init__(self, xq=XPT11, wq=XW11, jquad=A.FJ_JQUAD_QAGS, precision=A.FJ_PREC_FP64):
        self.xq, self.wq = _f64(xq), _f64(wq)
        self.c = A.fj_quad_rule(len(self.xq), _dp(self.xq), _dp(self.wq), jquad, precision)


class DeviceTables:
    """A C-ABI struct of device pointers together with the tensors that own the memory
    (the struct alone would let the caching allocator reuse it under a queued kernel)."""

    def __init__(self, c, owners):
        self.c = c
        self.owners = owners


class Context:
    """One CUDA context/stream of libfjgpu (fj_ctx)."""

    def __init__(self, device=0):
        self.lib = A.load()
        h = C.c_void_p()
        rc = self.lib.fj_ctx_create(device, C.byref(h))
        if rc != A.FJ_OK:
            raise FJError(f"fj_ctx_create failed ({rc}): no usable CUDA device {device}")
        self.h = h

    def close(self):
        if self.h:
            self.lib.fj_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _on_torch_stream(self):
        """Order library work after torch's work on the current stream (where the
        tensors' copies were queued)."""
        import torch
        self.lib.fj_ctx_set_stream(self.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))

    def _check(self, rc, what):
        if rc != A.FJ_OK:
            raise FJError(f"{what} failed ({rc}): {self.lib.fj_last_error(self.h).decode()}")

    def sync(self):
        self._check(self.lib.fj_ctx_synchronize(self.h), "synchronize")

    def use_own_stream(self):
        self.lib.fj_ctx_set_stream(self.h, self.lib.fj_ctx_own_stream(self.h))

    # ---------------------------------------------------------------- structs
    @staticmethod
    def potential(ar, phil, Pr, Pr2):
        """Device multipole potential; the returned object keeps the tensors alive."""
        return DeviceTables(A.fj_potential(ar.numel(), phil.numel() // ar.numel(), _ptr(ar), _ptr(phil), _ptr(Pr),
                                           _ptr(Pr2)), (ar, phil, Pr, Pr2))

    @staticmethod
    def delta(Egrid, Dgrid):
        """Device focal-distance table; the returned object keeps the tensors alive."""
        return DeviceTables(A.fj_delta_table(Egrid.numel(), _ptr(Egrid), _ptr(Dgrid)), (Egrid, Dgrid))

    # ---------------------------------------------------------------- hot path
    def moments(self, pot, delta, df, rule, ngauss, grids6):
        """rhofDF over the meridional grid (pot/potLeg.cpp:54-58)."""
        self._on_torch_stream()
        st = A.fj_moment_stats()
        self._check(self.lib.fj_moments(self.h, C.byref(pot.c), C.byref(delta.c), C.byref(df.c), C.byref(rule.c),
                                        ngauss, _ptr(grids6), C.byref(st)), "fj_moments")
        return st

    def moments_points(self, pot, delta, df, rule, Rz, out6):
        self._on_torch_stream()
        st = A.fj_moment_stats()
        self._check(self.lib.fj_moments_points(self.h, C.byref(pot.c), C.byref(delta.c), C.byref(df.c),
                                               C.byref(rule.c), _ptr(Rz), Rz.shape[0], _ptr(out6), C.byref(st)),
                    "fj_moments_points")
        return st

    def moments_batch(self, items, rule):
        """Many models' moment grids in one launch; items = [(pot, delta, df, ngauss, grids6)]
        with pot/delta from potential()/delta() and grids6 device [6][nr*ngauss]."""
        self._on_torch_stream()
        arr = (A.fj_batch_item * len(items))()
        for i, (pot, delta, df, ng, grids) in enumerate(items):
            arr[i] = A.fj_batch_item(pot.c, delta.c, df.c, ng, _ptr(grids))
        st = A.fj_moment_stats()
        self._check(self.lib.fj_moments_batch(self.h, len(items), arr, C.byref(rule.c), C.byref(st)),
                    "fj_moments_batch")
        return st

    def set_action_output(self, jout):
        """Mixed form: write every bound node's (Jr, Jz) into jout (device f32 [npts][nq^3][2]); None: off."""
        self._check(self.lib.fj_set_action_output(self.h, _ptr(jout) if jout is not None else None),
                    "fj_set_action_output")

    def run_model_surrogate(self, nr, ngauss, npoly, rmin, rmax, df, rule, itermax, surrogate, tol=0.0, ngrid=30,
                            q=1.0, delta_table=None, exact_first=1, exact_last=3, samples=1 << 20, epochs_first=8,
                            epochs=2, lr=1e-3, seed=1, r_exact=None, audit_stride=100, audit_tol=1e-2):
        """The self-consistent loop with the action surrogate in the middle iterations
        (fj_run_model_surrogate); returns (result dict as run_model, report dict)."""
        self.use_own_stream()
        din = [None, None] if delta_table is None else [_f64(delta_table[0]), _f64(delta_table[1])]
        cfg = A.fj_model_config(nr, ngauss, npoly, ngrid, rmin, rmax, A.FJ_GUESS.get(df.model, 0), df.mass, df.r0,
                                q, df.c, rule.c, itermax, tol, *[_dp(d) if d is not None else None for d in din])
        sch = A.fj_surrogate_schedule(exact_first, exact_last, samples, epochs_first, epochs, lr, seed,
                                      0.05 * df.r0 if r_exact is None else r_exact, audit_stride, audit_tol)
        out = {"ar": np.zeros(nr), "coef6": np.zeros((6, nr, npoly)), "phil": np.zeros((nr, npoly)),
               "Pr": np.zeros((nr, npoly)), "Pr2": np.zeros((nr, npoly)), "Egrid": np.zeros(ngrid),
               "Dgrid": np.zeros(ngrid), "grids6": np.zeros((6, nr, ngauss))}
        res = A.fj_model_result(*[_dp(out[k]) for k in ("ar", "coef6", "phil", "Pr", "Pr2", "Egrid", "Dgrid",
                                                        "grids6")])
        rep = A.fj_surrogate_report()
        self._check(self.lib.fj_run_model_surrogate(self.h, C.byref(cfg), C.byref(sch), surrogate.h, C.byref(res),
                                                    C.byref(rep)), "fj_run_model_surrogate")
        out.update(vir7=np.array(res.vir7[:]), iterations=res.iterations, last_change=res.last_change,
                   bound=res.bound, failures=res.failures, wall_ms=res.wall_ms, kernel_ms=res.kernel_ms,
                   setup_ms=res.setup_ms)
        return out, {f: getattr(rep, f) for f, _ in A.fj_surrogate_report._fields_}

    def run_model_batch(self, models, rule, itermax, tol=0.0, ngrid=30, use_graph=True, delta_gpu=False,
                        delta_every=0):
        """Several one-component models iterated together (fj_run_model_batch).  models = list of
        dicts with nr, ngauss, npoly, rmin, rmax, df (DFParams) and optional q, delta_table, and
        df2 (+ q2) for a second component (summed order, as run_model's FJ_TWOCOMP_SUMMED).
        delta_gpu: focal-distance tables on the GPU, all models in one launch; delta_every = 1
        tabulates them again before every later iteration."""
        self.use_own_stream()
        n = len(models)
        cfgs = (A.fj_model_config * n)()
        ress = (A.fj_model_result * n)()
        keep, outs = [], []
        for i, m in enumerate(models):
            nr, ng, npl, df = m["nr"], m["ngauss"], m["npoly"], m["df"]
            dt = m.get("delta_table")
            din = [None, None] if dt is None else [_f64(dt[0]), _f64(dt[1])]
            keep.append(din)
            cfgs[i] = A.fj_model_config(nr, ng, npl, ngrid, m["rmin"], m["rmax"], A.FJ_GUESS.get(df.model, 0), df.mass,
                                        df.r0, m.get("q", 1.0), df.c, rule.c, itermax, tol,
                                        *[_dp(d) if d is not None else None for d in din])
            cfgs[i].delta_gpu, cfgs[i].delta_every = int(delta_gpu), int(delta_every)
            df2 = m.get("df2")
            if df2 is not None:
                c = cfgs[i]
                c.ncomp, c.guess2, c.mass2, c.r0_2, c.q2 = 2, A.FJ_GUESS.get(df2.model, 0), df2.mass, df2.r0, m.get("q2", 1.0)
                c.df2, c.twocomp_order = df2.c, A.FJ_TWOCOMP_SUMMED
            out = {"ar": np.zeros(nr), "coef6": np.zeros((6, nr, npl)), "phil": np.zeros((nr, npl)),
                   "Pr": np.zeros((nr, npl)), "Pr2": np.zeros((nr, npl)), "Egrid": np.zeros(ngrid),
                   "Dgrid": np.zeros(ngrid)}
            outs.append(out)
            ress[i] = A.fj_model_result(*[_dp(out[k]) for k in ("ar", "coef6", "phil", "Pr", "Pr2", "Egrid",
                                                                  "Dgrid")], None)
            if df2 is not None:
                out["coef6_2"] = np.zeros((6, nr, npl))
                ress[i].coef6_2 = _dp(out["coef6_2"])
        self._check(self.lib.fj_run_model_batch(self.h, n, cfgs, ress, 1 if use_graph else 0), "fj_run_model_batch")
        for out, r in zip(outs, ress):
            out.update(vir7=np.array(r.vir7[:]), iterations=r.iterations, last_change=r.last_change, bound=r.bound,
                       failures=r.failures, wall_ms=r.wall_ms, kernel_ms=r.kernel_ms, setup_ms=r.setup_ms)
            if "coef6_2" in out:
                out["vir7_2"] = np.array(r.vir7_2[:])
        return outs

    def tabulate_delta_batch(self, pots, ngrid=30):
        """Focal-distance tables of several models on the GPU (fj_tabulate_delta_batch); pots from
        potential().  Returns device (Egrid, Dgrid) [n][ngrid] and the per-model status list."""
        import torch
        self._on_torch_stream()
        n = len(pots)
        arr = (A.fj_potential * n)(*[p.c for p in pots])
        E = torch.zeros((n, ngrid), dtype=torch.float64, device="cuda")
        D = torch.zeros_like(E)
        st = (C.c_int * n)()
        self._check(self.lib.fj_tabulate_delta_batch(self.h, n, arr, ngrid, _ptr(E), _ptr(D), st),
                    "fj_tabulate_delta_batch")
        return E, D, list(st)

    def tc_gemm(self, a, b, c, ksplit=1):
        """c = a @ b.T on the tensor cores: a [M][K], b [N][K] bfloat16, c [M][N] float32 (device)."""
        import torch
        m, k = a.shape
        n = b.shape[0]
        rc = self.lib.fj_tc_gemm(m, n, k, _ptr(a), a.stride(0), _ptr(b), b.stride(0), _ptr(c), c.stride(0), ksplit,
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
        if rc != A.FJ_OK:
            raise FJError(f"fj_tc_gemm failed ({rc})")

    def set_mixed_config(self, variant, nodes_per_block):
        self._check(self.lib.fj_set_mixed_config(self.h, variant, nodes_per_block), "fj_set_mixed_config")

    def set_poisson(self, mode):
        """Radial integrals of every Poisson solve on this context: A.FJ_POISSON_QAGS (the
        reference's adaptive quadrature, the default) or A.FJ_POISSON_CUMULATIVE (exact
        interval integrals of the same integrands, prefix-summed)."""
        self._check(self.lib.fj_set_poisson(self.h, mode), "fj_set_poisson")

    def poisson(self):
        m = C.c_int()
        self._check(self.lib.fj_get_poisson(self.h, C.byref(m)), "fj_get_poisson")
        return m.value

    def mixed_config(self):
        v, c = C.c_int(), C.c_int()
        self._check(self.lib.fj_get_mixed_config(self.h, C.byref(v), C.byref(c)), "fj_get_mixed_config")
        return v.value, c.value

    def autotune_mixed(self, pot, delta, df, rule, Rz):
        """Time the mixed kernel's configurations on sample points Rz [n][2] (device) and keep
        the fastest; returns (variant, nodes_per_block, kernel_ms)."""
        import torch
        self._on_torch_stream()
        out = torch.zeros((6, Rz.shape[0]), dtype=torch.float64, device=Rz.device)
        ms = np.zeros(1)
        self.autotune_table = np.zeros((8, 3))
        self._check(self.lib.fj_autotune_mixed(self.h, C.byref(pot.c), C.byref(delta.c), C.byref(df.c),
                                               C.byref(rule.c), _ptr(Rz), Rz.shape[0], _ptr(out), _dp(ms),
                                               _dp(self.autotune_table)), "fj_autotune_mixed")
        return (*self.mixed_config(), float(ms[0]))

    def legendre_project(self, nr, ngauss, npoly, ar, grids6, coef6):
        self._on_torch_stream()
        self._check(self.lib.fj_legendre_project(self.h, nr, ngauss, npoly, _ptr(ar), _ptr(grids6), _ptr(coef6)),
                    "fj_legendre_project")

    def computePhil(self, ar, rhl, phil, Pr, Pr2):
        self._on_torch_stream()
        nr = ar.numel()
        self._check(self.lib.fj_poisson(self.h, nr, rhl.numel() // nr, _ptr(ar), _ptr(rhl), _ptr(phil), _ptr(Pr),
                                        _ptr(Pr2)), "fj_poisson")

    def updatePhil(self, a3, b3, out3):
        self._on_torch_stream()
        n = a3[0].numel()
        self._check(self.lib.fj_sum_potentials(self.h, n, *[_ptr(t) for t in (*a3, *b3, *out3)]),
                    "fj_sum_potentials")

    def computeNewPhi(self, pot, delta, df, rule, ngauss, grids6, coef6, phil, Pr, Pr2):
        self._on_torch_stream()
        st = A.fj_moment_stats()
        self._check(self.lib.fj_compute_new_phi(self.h, C.byref(pot.c), C.byref(delta.c), C.byref(df.c),
                                                C.byref(rule.c), ngauss, _ptr(grids6), _ptr(coef6), _ptr(phil),
                                                _ptr(Pr), _ptr(Pr2), C.byref(st)), "fj_compute_new_phi")
        return st

    def uvOrb_actions(self, pot, delta, pts, out, jquad=A.FJ_JQUAD_QAGS):
        self._on_torch_stream()
        self._check(self.lib.fj_actions(self.h, C.byref(pot.c), C.byref(delta.c), _ptr(pts), pts.shape[0], jquad,
                                        _ptr(out)), "fj_actions")

    def potential_eval(self, pot, Rz, out):
        self._on_torch_stream()
        self._check(self.lib.fj_potential_eval(self.h, C.byref(pot.c), _ptr(Rz), Rz.shape[0], _ptr(out)),
                    "fj_potential_eval")

    def los(self, pot, delta, df, rule, rhl, kind, Rzv, out):
        """SigmaDF / line_profile / P_vp / P_vz / P_vr (integ/Integ.cpp:168-220) at Rzv (device
        [n][3] = R, z, v) into out (device [n]); rhl device [nr][npoly] density multipoles
        (needed by SIGMA and LINE, else may be None).  Returns the fj_moment_stats."""
        self._on_torch_stream()
        st = A.fj_moment_stats()
        self._check(self.lib.fj_los(self.h, C.byref(pot.c), C.byref(delta.c), C.byref(df.c), C.byref(rule.c),
                                    _ptr(rhl) if rhl is not None else None, kind, _ptr(Rzv), Rzv.shape[0],
                                    _ptr(out), C.byref(st)), "fj_los")
        return st

    def line_profile_file(self, path, pot, delta, df, rule, rhl, size_lp=150):
        """The line-profile file of writeOut (io/writeOut.cpp:159-187, its LINEPROFILE block):
        size_lp rows of (vx, line profile) at the centre (ar[0], ar[0]), at ar[2 nr/3] and at
        ar[5 nr/6] (z = ar[0]), vx = 3 v_i on a signed log grid in units of each point's
        escape speed, the first column of each pair scaled by it.  pot's tables on the device."""
        import torch
        ar = pot.owners[0].cpu().numpy()
        nr = len(ar)
        rmax = ar[-1]
        pts = torch.tensor([[ar[0], ar[0]], [ar[nr * 2 // 3], ar[0]], [ar[nr * 5 // 6], ar[0]],
                            [10 * rmax, 10 * rmax]], dtype=torch.float64, device="cuda")
        ph = torch.zeros((4, 3), dtype=torch.float64, device="cuda")
        self.potential_eval(pot, pts, ph)
        phi = ph[:, 0].cpu().numpy()
        ve = np.sqrt(-2 * (phi[:3] - phi[3]))
        half = size_lp // 2
        v = np.zeros(size_lp)
        for i in range(half):
            v[i] = -10.0 ** (-3.0 + (half - 1 - i) * 3.0 / (half - 1))
        for i in range(half, size_lp):
            v[i] = 10.0 ** (-3.0 + (i - half) * 3.0 / (half - 1))
        Rz = [(ar[0], ar[0]), (ar[nr * 2 // 3], ar[0]), (ar[nr * 5 // 6], ar[0])]
        rzv = torch.tensor([[R, z, 3.0 * vi] for R, z in Rz for vi in v], dtype=torch.float64, device="cuda")
        out = torch.zeros(rzv.shape[0], dtype=torch.float64, device="cuda")
        self.los(pot, delta, df, rule, rhl, A.FJ_LOS_LINE, rzv, out)
        lp = out.cpu().numpy().reshape(3, size_lp)
        with open(path, "w") as f:
            for i in range(size_lp):
                f.write(" ".join(f"{x:g}" for x in (ve[0] * 3.0 * v[i], lp[0, i], ve[1] * 3.0 * v[i], lp[1, i],
                                                    ve[2] * 3.0 * v[i], lp[2, i])) + "\n")
        return lp

    def vir2(self, pot, ngauss, coef6):
        self._on_torch_stream()
        out = np.zeros(7)
        self._check(self.lib.fj_vir2(self.h, C.byref(pot.c), ngauss, _ptr(coef6), _dp(out)), "fj_vir2")
        return dict(zip(("KRR", "Kzz", "WRR", "Wzz", "pot", "mass_pr", "mass_sum"), out))

    # ---------------------------------------------------------------- whole model
    def anderson_reset(self, depth, beta=1.0):
        """Start a new mixed iteration with history depth m and mixing factor beta
        (fj_anderson_reset; depth 0 = plain steps)."""
        self._check(self.lib.fj_anderson_reset(self.h, int(depth), float(beta)), "fj_anderson_reset")

    def anderson_step(self, x, g):
        """One Anderson step (fj_anderson_step): x, g are contiguous device tensors [3][nr][npoly]
        (phil, Pr, Pr2) of the last input and its computeNewPhi output; x is overwritten with the
        next input.  Returns the plain step's change max|dphil|/|phil(r, 0)|."""
        if x.shape != g.shape or x.dim() != 3 or x.shape[0] != 3 or not (x.is_contiguous() and g.is_contiguous()):
            raise FJError("anderson_step: x and g must be contiguous [3][nr][npoly] tensors")
        self._on_torch_stream()
        ch = np.zeros(1)
        self._check(self.lib.fj_anderson_step(self.h, x.shape[1], x.shape[2], _ptr(x), _ptr(g), _dp(ch)),
                    "fj_anderson_step")
        return float(ch[0])

    def run_model(self, nr, ngauss, npoly, rmin, rmax, df, rule, itermax, tol=0.0, ngrid=30, q=1.0,
                  keep_grids=False, delta_table=None, df2=None, q2=1.0, twocomp_order=A.FJ_TWOCOMP_SUMMED,
                  restart=None, delta_gpu=False, delta_every=0, ext=None, accel=0, accel_beta=1.0):
        """Self-consistent model (oneComp, fJmodels.cpp:86-144; with df2, the two-component
        loop of fJmodels.cpp:38-84 in `twocomp_order`) with host buffers.
        delta_table = (Egrid, Dgrid) uses a given focal-distance table instead of tabulating one;
        restart = a dict with ar, phil, Pr, Pr2 (readOut, or an earlier result) iterates on from
        those tables instead of the guess density (rmin, rmax are then unused).
        delta_gpu tabulates the focal-distance table on the GPU; delta_every = k > 0 tabulates it
        again from the new potential after every k-th iteration (the reference: once).
        ext = (phil, Pr, Pr2) of a fixed external potential added after the guess and after every
        iteration (the reference's external mode, fJmodels.cpp:120-125, 134).
        accel = m > 0 mixes each next input potential from the last m + 1 outputs (Anderson,
        mixing factor accel_beta; the reference iterates the plain map); with tol the loop then
        ends with a confirming plain step."""
        self.use_own_stream()
        din = [None, None] if delta_table is None else [_f64(delta_table[0]), _f64(delta_table[1])]
        cfg = A.fj_model_config(nr, ngauss, npoly, ngrid, rmin, rmax, A.FJ_GUESS.get(df.model, 0), df.mass, df.r0,
                                q, df.c, rule.c, itermax, tol, *[_dp(d) if d is not None else None for d in din])
        cfg.delta_gpu, cfg.delta_every, cfg.accel = int(delta_gpu), int(delta_every), int(accel)
        cfg.accel_beta = float(accel_beta)
        if ext is not None:
            ex = [_f64(t) for t in ext]
            if any(t.size != nr * npoly for t in ex):
                raise FJError("run_model: external potential tables do not match nr, npoly")
            cfg.ext_phil, cfg.ext_Pr, cfg.ext_Pr2 = (_dp(t) for t in ex)
        if restart is not None:
            rs = {k: _f64(restart[k]) for k in ("ar", "phil", "Pr", "Pr2")}
            if rs["ar"].size != nr or any(rs[k].size != nr * npoly for k in ("phil", "Pr", "Pr2")):
                raise FJError("run_model: restart tables do not match nr, npoly")
            cfg.ar_in, cfg.phil_in, cfg.Pr_in, cfg.Pr2_in = (_dp(rs[k]) for k in ("ar", "phil", "Pr", "Pr2"))
        if df2 is not None:
            cfg.ncomp, cfg.guess2, cfg.mass2, cfg.r0_2, cfg.q2 = 2, A.FJ_GUESS.get(df2.model, 0), df2.mass, df2.r0, q2
            cfg.df2 = df2.c
            cfg.twocomp_order = twocomp_order
        out = {"ar": np.zeros(nr), "coef6": np.zeros((6, nr, npoly)), "phil": np.zeros((nr, npoly)),
               "Pr": np.zeros((nr, npoly)), "Pr2": np.zeros((nr, npoly)), "Egrid": np.zeros(ngrid),
               "Dgrid": np.zeros(ngrid)}
        grids = np.zeros((6, nr, ngauss)) if keep_grids else None
        res = A.fj_model_result(*[_dp(out[k]) for k in ("ar", "coef6", "phil", "Pr", "Pr2", "Egrid", "Dgrid")],
                                _dp(grids) if keep_grids else None)
        if df2 is not None:
            out["coef6_2"] = np.zeros((6, nr, npoly))
            res.coef6_2 = _dp(out["coef6_2"])
        self._check(self.lib.fj_run_model(self.h, C.byref(cfg), C.byref(res)), "fj_run_model")
        if df2 is not None:
            out["vir7_2"] = np.array(res.vir7_2[:])
        out.update(vir7=np.array(res.vir7[:]), iterations=res.iterations, last_change=res.last_change,
                   bound=res.bound, failures=res.failures, wall_ms=res.wall_ms, kernel_ms=res.kernel_ms,
                   setup_ms=res.setup_ms)
        if keep_grids:
            out["grids6"] = grids
        return out


# -------------------------------------------------------------- host setup
def log_grid(rmin, rmax, n):
    ar = np.zeros(n)
    if A.load().fj_log_grid(rmin, rmax, n, _dp(ar)) != A.FJ_OK:
        raise FJError("log_grid: bad arguments")
    return ar


def tanh_sinh01():
    """The reference's 22-point tanh-sinh table on [0,1] (include/GaussPts.h:91-134)."""
    x = np.zeros(22)
    w = np.zeros(22)
    A.load().fj_tanh_sinh01(_dp(x), _dp(w))
    return x, w


def gauleg(x1, x2, n):
    x, w = np.zeros(n), np.zeros(n)
    A.load().fj_gauleg(x1, x2, n, _dp(x), _dp(w))
    return x, w


def guess_rhl(ar, ngauss, npoly, model="Hernquist", mass=1.0, r0=1.0, q=1.0):
    ar = _f64(ar)
    rhl = np.zeros((len(ar), npoly))
    if A.load().fj_guess_rhl(len(ar), ngauss, npoly, _dp(ar), A.FJ_GUESS[model], mass, r0, q, _dp(rhl)) != A.FJ_OK:
        raise FJError("guess_rhl: bad arguments")
    return rhl


def tabulate_delta(ar, phil, Pr, Pr2, ngrid=30):
    """tabulateDelta on host tables (delta/tabulate.cpp:13-38)."""
    ar, phil, Pr, Pr2 = (_f64(x) for x in (ar, phil, Pr, Pr2))
    pot = A.fj_potential(len(ar), phil.size // len(ar), ar.ctypes.data, phil.ctypes.data, Pr.ctypes.data,
                         Pr2.ctypes.data)
    E, D = np.zeros(ngrid), np.zeros(ngrid)
    rc = A.load().fj_tabulate_delta(C.byref(pot), ngrid, _dp(E), _dp(D))
    return E, D, rc


def writeOut(path, ar, mats9, ngauss, header, digits=0):
    """_writeOut (io/writeOut.cpp:74-138).  header = (dphi_h, dz_h, dphi_g, dz_g, chi, mass, r0, A, B).
    digits = 0 writes the reference's bytes; 17 writes every value exactly (a full-precision restart)."""
    ar = _f64(ar)
    m = _f64(mats9)
    nr = len(ar)
    npoly = m.size // (9 * nr)
    hdr = np.zeros(10)
    hdr[:9] = header
    rc = A.load().fj_write_out_digits(path.encode(), nr, npoly, ngauss, _dp(hdr), _dp(ar), _dp(m), digits)
    if rc != A.FJ_OK:
        raise FJError(f"writeOut failed ({rc}) for {path}")


OUT_TABLES = ("rhl", "vrotl", "sigRl", "sigpl", "sigzl", "sigRzl", "phil", "Pr", "Pr2")


def readOut(path):
    """A coefficient file of writeOut read back: dict with nr, npoly, ngauss, header (the nine
    values of writeOut's header), ar [nr] and the nine [nr][npoly] tables by their names
    (OUT_TABLES).  Its ar, phil, Pr and Pr2 restart a model: Context.run_model(restart=...)."""
    lib = A.load()
    nr, npoly, ngauss = C.c_int(), C.c_int(), C.c_int()
    hdr = np.zeros(10)
    rc = lib.fj_read_out(path.encode(), C.byref(nr), C.byref(npoly), C.byref(ngauss), _dp(hdr), None, None)
    if rc != A.FJ_OK:
        raise FJError(f"readOut failed ({rc}) for {path}")
    ar = np.zeros(nr.value)
    mats = np.zeros((9, nr.value, npoly.value))
    rc = lib.fj_read_out(path.encode(), C.byref(nr), C.byref(npoly), C.byref(ngauss), _dp(hdr), _dp(ar), _dp(mats))
    if rc != A.FJ_OK:
        raise FJError(f"readOut failed ({rc}) for {path}")
    out = {"nr": nr.value, "npoly": npoly.value, "ngauss": ngauss.value, "header": hdr[:9].copy(), "ar": ar}
    out.update({k: mats[i] for i, k in enumerate(OUT_TABLES)})
    return out


def _to_string(x, eps=2):
    return f"{x:.{eps}f}"


def composeName(model, dphi_h, dz_h, dphi_g, dz_g, it, comp=1, outName="null"):
    """Output file name of io/writeOut.cpp:22-56 and 87-88."""
    if outName != "null":
        name = f"{outName}_{it}.out"
    else:
        name = model[:5] + "_" + "_".join(_to_string(v) for v in (dphi_h, dz_h, dphi_g, dz_g)) + f"_{it}.out"
    if comp == 2 and outName == "null":
        name += "2c"
    return os.path.join("models", name)


UNSET = -999.0


def readParam(path="param.txt"):
    """Key/value parameter file of io/readParam.cpp:31-111 (unknown keys ignored,
    comment/blank/indented lines skipped); returns (params dict, component count)."""
    keys = {"itermax": "itermax", "model": "modName", "A": "alpha", "B": "beta", "outfile": "outName",
            "chi": "chi", "h(J):dphi": "dphi_h_in", "h(J):dz": "dz_h_in", "g(J):dphi": "dphi_g_in",
            "g(J):dz": "dz_g_in", "mass": "mass", "r0": "r0", "q": "q"}
    p = {"itermax": 5, "modName": "null", "outName": "null"}
    for v in ("alpha", "beta", "dphi_h_in", "dz_h_in", "dphi_g_in", "dz_g_in", "chi", "mass", "r0", "q"):
        p[v] = UNSET
        p[v + "_2" if not v.endswith("_in") else v + "2"] = UNSET
    p["modName2"] = p["outName2"] = "null"
    if not os.path.exists(path):
        raise FJError(f"ERROR in opening parameter file {path}! Are you sure the file exists?")
    for line in open(path):
        line = line.rstrip("\n")
        if not line or line[0] in "# \t":
            continue
        parts = line.split()
        key, val = parts[0], (parts[1] if len(parts) > 1 else None)
        two = key.startswith("2:")
        base = key[2:] if two else key
        if base not in keys or val is None:
            continue
        field = keys[base]
        if two:
            field = {"modName": "modName2", "outName": "outName2"}.get(field, field + ("2" if field.endswith("_in") else "_2"))
        if field.startswith(("modName", "outName")):
            p[field] = val
        else:
            p[field] = int(float(val)) if field == "itermax" else float(val)
    one = ((p["modName"] != "null" or (p["alpha"] != UNSET and p["beta"] != UNSET)) and
           all(p[k] != UNSET for k in ("chi", "mass", "r0", "q", "dphi_h_in", "dz_h_in", "dphi_g_in", "dz_g_in")))
    if not one:
        raise FJError("ERROR: parameterfile must contain at least one component!")
    comps = 1
    if p["modName2"] != "null" or (p["alpha_2"] != UNSET and p["beta_2"] != UNSET):
        if all(p[k] != UNSET for k in ("chi_2", "mass_2", "r0_2", "q_2", "dphi_h_in2", "dz_h_in2", "dphi_g_in2",
                                        "dz_g_in2")):
            comps = 2
        else:
            raise FJError("ERROR in parameterfile: second components is missing some parameter to initialize!")
    return p, comps


class Anderson:
    """Anderson mixing of a self-consistent loop on host tables (fj_anderson_create /
    fj_anderson_host_step; no device work): depth m, mixing factor beta.  step(x, g) takes
    float64 arrays [3][nr][npoly] (phil, Pr, Pr2) of the last input and its output, overwrites
    x with the next input and returns the plain step's change max|dphil| / |phil(r, 0)|."""

    def __init__(self, depth, beta=1.0):
        self.lib = A.load()
        h = C.c_void_p()
        rc = self.lib.fj_anderson_create(int(depth), float(beta), C.byref(h))
        if rc != A.FJ_OK:
            raise FJError(f"fj_anderson_create: depth in [0, {A.FJ_ANDERSON_MAX_DEPTH}] and beta in (0, 4]")
        self.h = h

    def step(self, x, g):
        if not (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous and x.ndim == 3
                and x.shape[0] == 3):
            raise FJError("Anderson.step: x must be a contiguous float64 array [3][nr][npoly]")
        g = _f64(g)
        if g.shape != x.shape:
            raise FJError("Anderson.step: x and g differ in shape")
        ch = np.zeros(1)
        rc = self.lib.fj_anderson_host_step(self.h, x.shape[1], x.shape[2], _dp(x), _dp(g), _dp(ch))
        if rc != A.FJ_OK:
            raise FJError(f"fj_anderson_host_step failed ({rc})")
        return float(ch[0])

    def close(self):
        if self.h:
            self.lib.fj_anderson_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Surrogate:
    """The action surrogate (fj_surrogate_*): MLP 16 -> 128 x 4 (GELU) -> 16 on the tensor
    cores, outputs 0 and 1 = (log Jr, log Jz) of normalised features."""

    LAYERS = [(128, 16), (128, 128), (128, 128), (128, 128), (16, 128)]  # (rows, cols) of W

    def __init__(self, ctx, batch=4096, seed=1):
        self.ctx, self.lib, self.batch = ctx, ctx.lib, batch
        h = C.c_void_p()
        ctx._on_torch_stream()
        rc = self.lib.fj_surrogate_create(ctx.h, batch, seed, C.byref(h))
        if rc != A.FJ_OK:
            raise FJError(f"fj_surrogate_create failed ({rc})")
        self.h = h
        self.nparam = self.lib.fj_surrogate_nparam(h)

    def close(self):
        if self.h:
            self.lib.fj_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _rc(self, rc, what):
        if rc != A.FJ_OK:
            raise FJError(f"{what} failed ({rc})")

    def params(self):
        p = np.zeros(self.nparam)
        self._rc(self.lib.fj_surrogate_params(self.h, _dp(p), None), "fj_surrogate_params")
        return p

    def set_params(self, p):
        p = _f64(p)
        self._rc(self.lib.fj_surrogate_params(self.h, None, _dp(p)), "fj_surrogate_params")

    def unpack(self, p):
        """[(W [rows][cols], b [rows])] per layer from a flat parameter vector."""
        out, o = [], 0
        for r, c in self.LAYERS:
            W = p[o:o + r * c].reshape(r, c)
            o += r * c
            out.append((W, p[o:o + r]))
            o += r
        return out

    def gradients(self, X, T):
        g, loss = np.zeros(self.nparam), np.zeros(1)
        self._rc(self.lib.fj_surrogate_gradients(self.h, _ptr(X), _ptr(T), _dp(g), _dp(loss)),
                 "fj_surrogate_gradients")
        return g, float(loss[0])

    def train(self, X, T, epochs=1, lr=1e-3):
        loss = np.zeros(1)
        self._rc(self.lib.fj_surrogate_train(self.h, _ptr(X), _ptr(T), X.shape[0], epochs, lr, _dp(loss)),
                 "fj_surrogate_train")
        return float(loss[0])

    def fit(self, pot, df, ngauss, rule, jout, samples, seed=1, epochs=1, lr=1e-3, rho=None):
        loss = np.zeros(1)
        self._rc(self.lib.fj_surrogate_fit(self.h, C.byref(pot.c), C.byref(df.c), ngauss, C.byref(rule.c),
                                           _ptr(jout), _ptr(rho) if rho is not None else None, samples, seed, epochs,
                                           lr, _dp(loss)), "fj_surrogate_fit")
        return float(loss[0])

    def moments(self, pot, df, rule, ngauss, grids6, fused=True):
        ms = np.zeros(1)
        self._rc(self.lib.fj_surrogate_moments(self.h, C.byref(pot.c), C.byref(df.c), C.byref(rule.c), ngauss,
                                               _ptr(grids6), _dp(ms), 1 if fused else 0), "fj_surrogate_moments")
        return float(ms[0])

    def predict(self, X, Y):
        self._rc(self.lib.fj_surrogate_predict(self.h, _ptr(X), X.shape[0], _ptr(Y)), "fj_surrogate_predict")

