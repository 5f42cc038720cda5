"""ctypes front end of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  Never imported by the product
package.  The C sources restate the reference algorithm; see fjoracle.h.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

DF_DPL = 0
DF_QUASIISO = 1

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

DP = C.POINTER(C.c_double)


class _Model(C.Structure):
    _fields_ = [("nr", C.c_int), ("npoly", C.c_int), ("ngauss", C.c_int), ("ngrid", C.c_int),
                ("ar", DP), ("phil", DP), ("Pr", DP), ("Pr2", DP), ("Egrid", DP), ("Dgrid", DP),
                ("df_kind", C.c_int),
                ("alpha", C.c_double), ("beta", C.c_double), ("J0", C.c_double), ("mass", C.c_double),
                ("dphi_h", C.c_double), ("dz_h", C.c_double), ("dphi_g", C.c_double), ("dz_g", C.c_double),
                ("chi", C.c_double), ("k", C.c_double),
                ("nq", C.c_int), ("xq", DP), ("wq", DP), ("jquad", C.c_int)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_longlong) for n in
                ("nodes", "bound", "phi_evals", "grad_evals", "brent_iters", "quad_evals", "failures")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


FN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)


def build(force=False):
    so = os.path.join(_HERE, "liboracle.so")
    if force or not os.path.exists(so) or any(
            os.path.getmtime(os.path.join(_HERE, f)) > os.path.getmtime(so)
            for f in os.listdir(_HERE) if f.endswith((".c", ".h"))):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return so


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(build())
        M = C.POINTER(_Model)
        S = C.POINTER(Stats)
        L.orc_gauleg.argtypes = [C.c_double, C.c_double, C.c_int, DP, DP]
        L.orc_brent_wrapped.argtypes = [FN, C.c_void_p, C.c_double, C.c_double, DP]
        L.orc_qags.argtypes = [FN, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, DP, DP]
        L.orc_qagiu.argtypes = [FN, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int, DP, DP]
        L.orc_evenlegend.argtypes = [C.c_int, C.c_double, DP]
        for fn in ("orc_phi", "orc_dR", "orc_dz"):
            getattr(L, fn).argtypes = [M, C.c_double, C.c_double]
            getattr(L, fn).restype = C.c_double
        L.orc_getfreqs.argtypes = [M, C.c_double, DP, DP, DP]
        L.orc_log_grid.argtypes = [C.c_double, C.c_double, C.c_int, DP]
        L.orc_deltafn.argtypes = [M, C.c_double]
        L.orc_deltafn.restype = C.c_double
        L.orc_actions.argtypes = [M, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.c_double, DP, DP, S]
        L.orc_df.argtypes = [M, C.c_double, C.c_double, C.c_double, DP, S]
        L.orc_df.restype = C.c_double
        L.orc_rhofDF.argtypes = [M, C.c_double, C.c_double, DP, S]
        L.orc_rhofDF.restype = C.c_double
        L.orc_moment_grid.argtypes = [M, C.c_int, C.c_int, DP, C.c_int, S]
        L.orc_project6.argtypes = [C.c_int, C.c_int, C.c_int, DP, DP, DP]
        L.orc_compute_phil.argtypes = [C.c_int, C.c_int, DP, DP, DP, DP, DP]
        L.orc_compute_phil_cumulative.argtypes = [C.c_int, C.c_int, DP, DP, DP, DP, DP]
        L.orc_guess_rhl.argtypes = [C.c_int, C.c_int, C.c_int, DP, C.c_int, C.c_double, C.c_double,
                                    C.c_double, DP]
        L.orc_vir2.argtypes = [M, DP, DP]
        L.orc_merge_distance.argtypes = [C.c_int, C.c_int, DP, DP]
        L.orc_merge_distance.restype = C.c_double
        L.orc_tabulate_delta.argtypes = [M, DP, DP]
        L.orc_tanh_sinh01.argtypes = [DP, DP]
        L.orc_los.argtypes = [M, DP, C.c_int, C.c_double, C.c_double, C.c_double, DP, DP, S]
        L.orc_los.restype = C.c_double
        _LIB = L
    return _LIB


def _p(a):
    return a.ctypes.data_as(DP)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


LOS_SIGMA, LOS_LINE, LOS_PVPHI, LOS_PVZ, LOS_PVR = range(5)


def tanh_sinh01():
    """The reference's 22-point tanh-sinh table on [0,1] (include/GaussPts.h:91-134)."""
    x = np.zeros(22)
    w = np.zeros(22)
    lib().orc_tanh_sinh01(_p(x), _p(w))
    return x, w


def gauleg(x1, x2, n):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().orc_gauleg(x1, x2, n, _p(x), _p(w))
    return x, w


def log_grid(rmin, rmax, n):
    ar = np.zeros(n)
    lib().orc_log_grid(rmin, rmax, n, _p(ar))
    return ar


def brent(f, lo, hi):
    cb = FN(lambda x, _: f(x))
    r = C.c_double()
    st = lib().orc_brent_wrapped(cb, None, lo, hi, C.byref(r))
    return r.value, st


def qags(f, a, b, epsabs=1e-5, epsrel=1e-3, limit=1000):
    cb = FN(lambda x, _: f(x))
    r, e = C.c_double(), C.c_double()
    st = lib().orc_qags(cb, None, a, b, epsabs, epsrel, limit, C.byref(r), C.byref(e))
    return r.value, e.value, st


def qagiu(f, a, epsabs=1e-4, epsrel=1e-3, limit=1000):
    cb = FN(lambda x, _: f(x))
    r, e = C.c_double(), C.c_double()
    st = lib().orc_qagiu(cb, None, a, epsabs, epsrel, limit, C.byref(r), C.byref(e))
    return r.value, e.value, st


class Model:
    """Inputs of one component: grid, potential multipoles, Delta table, DF parameters, rules."""

    def __init__(self, ar, phil, Pr, Pr2, Egrid, Dgrid, ngauss, *, df_kind=DF_DPL, alpha=1.667, beta=5.0,
                 mass=1.0, r0=1.0, dphi_h=0.55, dz_h=0.55, dphi_g=1.0, dz_g=1.0, chi=0.0, k=0.5,
                 xq=XPT11, wq=XW11, jquad=0):
        self.ar = _f64(ar)
        self.nr = len(self.ar)
        self.phil, self.Pr, self.Pr2 = (_f64(t).reshape(self.nr, -1) for t in (phil, Pr, Pr2))
        self.npoly = self.phil.shape[1]
        self.Egrid, self.Dgrid = _f64(Egrid), _f64(Dgrid)
        self.ngauss = ngauss
        self.xq, self.wq = _f64(xq), _f64(wq)
        self.params = dict(df_kind=df_kind, alpha=alpha, beta=beta, J0=float(np.sqrt(mass * r0)), mass=mass,
                           dphi_h=dphi_h, dz_h=dz_h, dphi_g=dphi_g, dz_g=dz_g, chi=chi, k=k)
        self.jquad = jquad

    def c(self):
        m = _Model()
        m.nr, m.npoly, m.ngauss, m.ngrid = self.nr, self.npoly, self.ngauss, len(self.Egrid)
        m.ar, m.phil, m.Pr, m.Pr2 = _p(self.ar), _p(self.phil), _p(self.Pr), _p(self.Pr2)
        m.Egrid, m.Dgrid = _p(self.Egrid), _p(self.Dgrid)
        for k, v in self.params.items():
            setattr(m, k, v)
        m.nq, m.xq, m.wq, m.jquad = len(self.xq), _p(self.xq), _p(self.wq), self.jquad
        self._c = m
        return C.byref(m)

    def phi(self, R, z):
        return lib().orc_phi(self.c(), R, z)

    def dR(self, R, z):
        return lib().orc_dR(self.c(), R, z)

    def dz(self, R, z):
        return lib().orc_dz(self.c(), R, z)

    def deltafn(self, E):
        return lib().orc_deltafn(self.c(), E)

    def actions(self, R, z, vR, vphi, vz, Phi=None, Delta=None):
        if Phi is None:
            Phi = self.phi(R, z)
        if Delta is None:
            H = 0.5 * (vR * vR + vphi * vphi + vz * vz) + Phi
            Delta = self.deltafn(H)
        Jr, Jz = C.c_double(), C.c_double()
        st = Stats()
        lib().orc_actions(self.c(), Delta, R, z, Phi, vR, vphi, vz, C.byref(Jr), C.byref(Jz), C.byref(st))
        return Jr.value, Jz.value

    def rhofDF(self, R, z):
        mom = np.zeros(6)
        st = Stats()
        lib().orc_rhofDF(self.c(), R, z, _p(mom), C.byref(st))
        return mom, st.as_dict()

    def moment_grid(self, p0=0, p1=None, nthreads=None):
        npts = self.nr * self.ngauss
        p1 = npts if p1 is None else p1
        g = np.zeros((6, npts))
        st = Stats()
        lib().orc_moment_grid(self.c(), p0, p1, _p(g), nthreads or os.cpu_count(), C.byref(st))
        return g, st.as_dict()

    def vir2(self, coef6):
        out = np.zeros(7)
        c6 = _f64(coef6)
        lib().orc_vir2(self.c(), _p(c6), _p(out))
        return dict(zip(("KRR", "Kzz", "WRR", "Wzz", "pot", "mass_pr", "mass_sum"), out))

    def los(self, rhl, kind, R, z, v=0.0):
        """SigmaDF / line_profile / P_vp / P_vz / P_vr (integ/Integ.cpp:168-220) at one (R, z, v);
        rhl [nr][npoly] density multipoles (SigmaDF); the model's rule is the [-1,1] rule."""
        x01, w01 = tanh_sinh01()
        r = _f64(rhl)
        return lib().orc_los(self.c(), _p(r), kind, R, z, v, _p(x01), _p(w01), None)

    def tabulate_delta(self, ngrid=30):
        E = np.zeros(ngrid)
        D = np.zeros(ngrid)
        saveE, saveD = self.Egrid, self.Dgrid
        self.Egrid, self.Dgrid = E, D
        fail = lib().orc_tabulate_delta(self.c(), _p(E), _p(D))
        self.Egrid, self.Dgrid = saveE, saveD
        return E.copy(), D.copy(), fail


_FLIB = None


def flop_counts(model, points):
    """The reference's algorithm with its floating-point operations tallied (liboracle_flops.so,
    orc_flops.cpp): the moments of the grid points `points` (indices p = n*ngauss + g) of
    `model`, one host thread.  Returns (moments [6][npts] for those points, counts dict add, mul,
    div, sqrt, trans); the moments are the oracle's bit for bit."""
    global _FLIB
    if _FLIB is None:
        so = os.path.join(_HERE, "liboracle_flops.so")
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle_flops.so"], check=True)
        L = C.CDLL(so)
        L.orc_moment_grid.argtypes = [C.POINTER(_Model), C.c_int, C.c_int, DP, C.c_int, C.POINTER(Stats)]
        L.orc_flops_reset.argtypes = []
        L.orc_flops_get.argtypes = [C.POINTER(C.c_ulonglong)]
        _FLIB = L
    L = _FLIB
    npts = model.nr * model.ngauss
    out = np.zeros((6, npts))
    mc = model.c()
    L.orc_flops_reset()
    for p in points:
        L.orc_moment_grid(mc, int(p), int(p) + 1, out.ctypes.data_as(DP), 1, C.byref(Stats()))
    cnt = (C.c_ulonglong * 5)()
    L.orc_flops_get(cnt)
    return out[:, list(points)], dict(zip(("add", "mul", "div", "sqrt", "trans"), [int(v) for v in cnt]))


def project6(ar, ngauss, npoly, grids6):
    nr = len(ar)
    g = _f64(grids6).copy()
    coef = np.zeros((6, nr * npoly))
    lib().orc_project6(nr, ngauss, npoly, _p(_f64(ar)), _p(g), _p(coef))
    return coef, g


def compute_phil(ar, rhl, cumulative=False):
    """Poisson solve: the reference's adaptive QAGS/QAGIU, or (cumulative=True) the same
    integrands integrated interval by interval without adaptivity."""
    ar = _f64(ar)
    rhl = _f64(rhl)
    nr, npoly = rhl.shape
    phil, Pr, Pr2 = np.zeros((nr, npoly)), np.zeros((nr, npoly)), np.zeros((nr, npoly))
    fn = lib().orc_compute_phil_cumulative if cumulative else lib().orc_compute_phil
    fn(nr, npoly, _p(ar), _p(rhl), _p(phil), _p(Pr), _p(Pr2))
    return phil, Pr, Pr2


GUESS = {"Hernquist": 0, "Isochrone": 1, "NFW": 2}


def guess_rhl(ar, ngauss, npoly, model="Hernquist", mass=1.0, r0=1.0, q=1.0):
    ar = _f64(ar)
    rhl = np.zeros((len(ar), npoly))
    lib().orc_guess_rhl(len(ar), ngauss, npoly, _p(ar), GUESS[model], mass, r0, q, _p(rhl))
    return rhl


def merge_distance(phil_new, phil_old):
    a, b = _f64(phil_new), _f64(phil_old)
    return lib().orc_merge_distance(a.shape[0], a.shape[1], _p(a), _p(b))
