"""Known-answer tests of the oracle's numerics, independent of the reference:
Legendre recurrences, Gauss-Legendre nodes, QUADPACK QAGS/QAGIU against
scipy's QUADPACK, Brent, and the Poisson solve of analytic densities."""
import numpy as np
import pytest
from scipy import integrate, special

from oracle import oracle as O


def test_even_legendre_against_scipy():
    import ctypes as C
    L = O.lib()
    for c in (0.0, 0.3, -0.77, 0.999):
        pol = np.zeros(12)
        L.orc_evenlegend(12, c, pol.ctypes.data_as(O.DP))
        ref = [special.eval_legendre(2 * k, c) for k in range(12)]
        assert np.allclose(pol, ref, rtol=1e-12, atol=1e-14)


def test_gauleg_against_numpy():
    x, w = O.gauleg(0, 1, 30)
    xr, wr = np.polynomial.legendre.leggauss(30)
    assert np.allclose(x, (xr + 1) / 2, atol=1e-15)
    # the reference stops Newton at |dz| <= 3e-11 and takes the weight from the last derivative
    assert np.allclose(w, wr / 2, rtol=1e-9)


@pytest.mark.parametrize("f,a,b", [(np.sqrt, 0.0, 1.0), (lambda x: np.log(x) if x > 0 else 0.0, 0.0, 1.0),
                                   (lambda x: x ** -0.5 if x > 0 else 0.0, 0.0, 1.0),
                                   (lambda x: np.sin(50 * x) * x, 0.0, 3.0)])
def test_qags_matches_quadpack(f, a, b):
    r, e, st = O.qags(f, a, b, 1e-10, 1e-10, 1000)
    s = integrate.quad(f, a, b, epsabs=1e-10, epsrel=1e-10, limit=1000)
    assert st == 0 and r == pytest.approx(s[0], rel=1e-14, abs=1e-15)


def test_qagiu_matches_quadpack():
    f = lambda x: np.exp(-x) / (1 + x * x)  # noqa: E731
    r, e, st = O.qagiu(f, 0.5, 1e-10, 1e-10)
    s = integrate.quad(f, 0.5, np.inf, epsabs=1e-10, epsrel=1e-10)
    assert st == 0 and r == pytest.approx(s[0], rel=1e-14)


def test_brent_wrapper_rule():
    r, st = O.brent(lambda x: x ** 3 - 2, 0.0, 3.0)
    assert st == 0 and abs(r - 2 ** (1 / 3)) < 1e-8
    r, st = O.brent(lambda x: x - 1e-4, 0.0, 1.0)  # |f(lo)| < 5e-4: the end point is returned
    assert r == 0.0


# radial force dPhi/dr = G M(<r) / r^2 of the analytic models (G = M = r0 = 1)
@pytest.mark.parametrize("model,force", [
    ("Hernquist", lambda r: 1 / (r + 1) ** 2),
    ("Isochrone", lambda r: r / (np.sqrt(1 + r * r) * (1 + np.sqrt(1 + r * r)) ** 2)),
    ("NFW", lambda r: (np.log(1 + r) - r / (1 + r)) / r ** 2),
])
def test_poisson_of_analytic_densities_converges(model, force):
    errs = []
    for nr in (60, 240):
        ar = O.log_grid(1e-3, 200.0, nr)
        rhl = O.guess_rhl(ar, 10, 3, model)
        p, pr, _ = O.compute_phil(ar, rhl)
        sel = (ar > 0.05) & (ar < 20)
        errs.append(np.max(np.abs(pr[sel, 0] / force(ar[sel]) - 1)))
        assert np.max(np.abs(p[sel, 1:])) < 1e-6 * np.max(np.abs(p[sel, 0]))  # spherical: no l > 0 terms
    assert errs[1] < errs[0] / 4 and errs[1] < 5e-3  # linear interpolation of rho: ~second order


def test_fudge_actions_in_the_isochrone_potential():
    """Staeckel-fudge actions (uvOrb/uvOrb.cpp) in the isochrone potential (G = M = b = 1)
    against its analytic actions: Jr = 1/sqrt(-2E) - (L + sqrt(L^2 + 4))/2 and, the
    potential being spherical, Jz + |Lz| = L.  A spherical potential is separable in
    prolate-spheroidal coordinates only as the focal distance goes to zero, so the test
    passes a small one (0.01); what remains is the multipole potential's interpolation
    error (~2e-3 in Phi on this grid), 4e-4 of Jr + L measured, bound 1e-3."""
    ar = O.log_grid(1e-3, 200.0, 240)
    rhl = O.guess_rhl(ar, 10, 3, "Isochrone")
    phil, Pr, Pr2 = O.compute_phil(ar, rhl)
    m = O.Model(ar, phil, Pr, Pr2, np.zeros(30), np.zeros(30), 10, alpha=0.0, beta=5.0)
    rng = np.random.default_rng(3)
    for _ in range(12):
        R, z = rng.uniform(0.3, 3), rng.uniform(-1, 1)
        r = np.hypot(R, z)
        phi = -1 / (1 + np.sqrt(1 + r * r))
        vR, vp, vz = rng.uniform(-0.4, 0.4, 3) * np.sqrt(-2 * phi)
        E = 0.5 * (vR * vR + vp * vp + vz * vz) + phi
        L = np.linalg.norm(np.cross([R, 0, z], [vR, vp, vz]))
        Jr_an = 1 / np.sqrt(-2 * E) - 0.5 * (L + np.sqrt(L * L + 4))
        Jr, Jz = m.actions(R, z, vR, vp, vz, Delta=0.01)
        assert abs(Jr - Jr_an) < 1e-3 * (Jr_an + L), (R, z, vR, vp, vz, Jr, Jr_an)
        assert abs(Jz + abs(R * vp) - L) < 1e-3 * (Jr_an + L), (R, z, vR, vp, vz, Jz, L)


def test_cumulative_poisson_second_order_to_analytic_hernquist():
    """The cumulative solve integrates the interpolated density exactly, so its error
    against Phi = -M/(r + r0) is the interpolation's: it falls ~4x per doubling of the
    grid, where the adaptive solve stalls near its tolerance (epsabs 1e-4, epsrel 1e-3)."""
    errs, errs_qags = [], []
    for nr in (200, 400, 800):
        ar = O.log_grid(1e-3, 1000.0, nr)
        rhl = O.guess_rhl(ar, 8, 1, "Hernquist")
        an = -1 / (ar + 1)
        m = ar > 0.01
        cum = O.compute_phil(ar, rhl, cumulative=True)[0][:, 0]
        qg = O.compute_phil(ar, rhl)[0][:, 0]
        errs.append(np.max(np.abs(cum[m] - an[m]) / np.abs(an[m])))
        errs_qags.append(np.max(np.abs(qg[m] - an[m]) / np.abs(an[m])))
    assert 3.5 < errs[0] / errs[1] < 4.5 and 3.5 < errs[1] / errs[2] < 4.5, errs
    assert errs[2] < 4e-4 and errs_qags[2] > 1.5 * errs[2], (errs, errs_qags)


def test_cumulative_poisson_agrees_with_adaptive_to_its_tolerance():
    ar = O.log_grid(1e-3, 300.0, 80)
    for model in ("Hernquist", "NFW"):
        rhl = O.guess_rhl(ar, 40, 7, model)
        a = O.compute_phil(ar, rhl)[0]
        b = O.compute_phil(ar, rhl, cumulative=True)[0]
        d = np.max(np.abs(a - b) / np.abs(b[:, :1]))
        assert 1e-5 < d < 5e-3, (model, d)


def _header_numbers(path):
    import re
    txt = open(path).read()
    body = txt[txt.index("{"):]
    return np.array([float(x) for x in re.findall(r"-?\d+\.\d+(?:e-?\d+)?", body)])


def test_rk8pd_tableau_order_conditions_and_tables():
    """The Prince & Dormand RK8(7) tableau (the reference's orbit stepper, delta/Delta.cpp:
    59-60): row sums and every Butcher order condition (200 trees to order 8 for the
    8th-order weights, to order 7 for the embedded ones) hold to the rounding of its
    published rationals; the oracle's table and the library's table agree exactly."""
    import importlib.util
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("rk8pd_tableau", os.path.join(root, "oracle", "rk8pd_tableau.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    rows, d8, d7, d78 = mod.check()
    assert rows < 1e-16 and d8 < 1e-15 and d7 < 1e-15 and d78 > 1e-6
    a = _header_numbers(os.path.join(root, "oracle", "orc_rk8pd.h"))
    b = _header_numbers(os.path.join(root, "fjmodels_gb300", "csrc", "fj_rk8pd.h"))
    assert a.shape == b.shape == (13 + 13 * 12 + 13 + 13,) and np.array_equal(a, b)



def test_counting_oracle_is_the_oracle_bit_for_bit():
    """oracle/orc_flops.cpp (the oracle with every floating-point operation tallied, the
    source of the bench's algorithmic FLOPs) gives the oracle's moments bit for bit, and
    counts every kind of operation."""
    ar = O.log_grid(1e-2, 100.0, 12)
    rhl = O.guess_rhl(ar, 4, 3, "Hernquist")
    phil, Pr, Pr2 = O.compute_phil(ar, rhl)
    m = O.Model(ar, phil, Pr, Pr2, np.zeros(30), np.zeros(30), 4)
    E, D, _ = m.tabulate_delta(30)
    m.Egrid, m.Dgrid = E, D
    pts = [21]
    mom, counts = O.flop_counts(m, pts)
    grids, _ = m.moment_grid(pts[0], pts[0] + 1, nthreads=1)
    assert np.array_equal(mom, grids[:, pts])
    assert all(counts[k] > 0 for k in ("add", "mul", "div", "sqrt", "trans"))
    assert counts["mul"] > counts["div"] > counts["sqrt"]
