"""Two-component models (fJmodels.cpp:38-84): a Hernquist bulge (M = 0.1, r0 = 1)
inside an NFW halo (M = 1, r0 = 10), each with its own double-power-law DF.

One iteration of fj_run_model in both two-component orders against the oracle
composed the same way from its per-component pieces (guess densities, Poisson,
moment grids, projection).  Plain FP64 form, 1e-9 on the density and potential
multipoles (scaled by the shell's monopole).  The velocity rule is a 10-point
tanh-sinh rule per axis so that the oracle's grids take seconds.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402
from fjmodels_gb300 import _abi as A  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.helpers import rel_rows  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = 1e-9
NR, NG, NPL, RMIN, RMAX = 24, 8, 4, 0.01, 200.0


def components():
    bulge = F.DFParams("Hernquist", dphi_h=0.7, dz_h=0.5, dphi_g=1.0, dz_g=1.0, chi=0.0, mass=0.1, r0=1.0)
    halo = F.DFParams("NFW", dphi_h=0.55, dz_h=0.9, dphi_g=1.0, dz_g=1.0, chi=1.0, mass=1.0, r0=10.0, k=0.5)
    return bulge, halo


def oracle_model(ar, pot, E, D, df, x, w):
    a, b = F.api.MODEL_SLOPES[df.model]
    c = df.c
    return O.Model(ar, *pot, E, D, NG, alpha=a, beta=b, mass=df.mass, r0=df.r0, dphi_h=c.dphi_h, dz_h=c.dz_h,
                   dphi_g=c.dphi_g, dz_g=c.dz_g, chi=c.chi, k=c.k, xq=x, wq=w)


def oracle_coef(ar, pot, E, D, df, x, w):
    g, st = oracle_model(ar, pot, E, D, df, x, w).moment_grid()
    assert st["failures"] == 0
    coef, _ = O.project6(ar, NG, NPL, g)
    return coef.reshape(6, NR, NPL)


@pytest.mark.parametrize("order", [A.FJ_TWOCOMP_SUMMED, A.FJ_TWOCOMP_REFERENCE])
def test_two_components_one_iteration(ctx, order):
    bulge, halo = components()
    x, w = F.tanh_sinh_rule(10)
    ar = O.log_grid(RMIN, RMAX, NR)
    p1 = O.compute_phil(ar, O.guess_rhl(ar, NG, NPL, "Hernquist", 0.1, 1.0))
    p2 = O.compute_phil(ar, O.guess_rhl(ar, NG, NPL, "NFW", 1.0, 10.0))
    total = [a + b for a, b in zip(p1, p2)]
    E, D, _ = oracle_model(ar, total, np.zeros(30), np.zeros(30), bulge, x, w).tabulate_delta(30)

    out = ctx.run_model(NR, NG, NPL, RMIN, RMAX, bulge, F.Rule(x, w), itermax=1, delta_table=(E, D), df2=halo,
                        twocomp_order=order)
    assert out["iterations"] == 1 and out["failures"] == 0

    c1 = oracle_coef(ar, total, E, D, bulge, x, w)
    if order == A.FJ_TWOCOMP_SUMMED:
        c2 = oracle_coef(ar, total, E, D, halo, x, w)
        new = O.compute_phil(ar, c1[0] + c2[0])
    else:
        pot1 = O.compute_phil(ar, c1[0])
        c2 = oracle_coef(ar, pot1, E, D, halo, x, w)
        pot2 = O.compute_phil(ar, c2[0])
        new = [a + b for a, b in zip(pot1, pot2)]
    # in the reference's order the halo is evaluated in a potential solved from the bulge's
    # moments: their rounding-level differences (summation order) move the halo's adaptive
    # quadrature at ties, two chained parity steps, so its gate is 2 x TOL (1.3e-9 measured)
    tol2 = TOL if order == A.FJ_TWOCOMP_SUMMED else 2 * TOL
    for q in (0, 2, 3, 4):
        assert rel_rows(out["coef6"][q], c1[q]) < TOL, ("bulge", q)
        assert rel_rows(out["coef6_2"][q], c2[q]) < tol2, ("halo", q)
    assert rel_rows(out["phil"], new[0]) < tol2
    assert rel_rows(out["Pr"], new[1]) < tol2
    # both components' virial sums in the final total potential are reported
    assert np.all(np.isfinite(out["vir7"][:5])) and np.all(np.isfinite(out["vir7_2"][:5]))


def test_two_components_mixed_form(ctx):
    """The same two-component iteration in the mixed-precision form, within its 1e-4 gate."""
    bulge, halo = components()
    x, w = F.tanh_sinh_rule(10)
    ar = O.log_grid(RMIN, RMAX, NR)
    p1 = O.compute_phil(ar, O.guess_rhl(ar, NG, NPL, "Hernquist", 0.1, 1.0))
    p2 = O.compute_phil(ar, O.guess_rhl(ar, NG, NPL, "NFW", 1.0, 10.0))
    total = [a + b for a, b in zip(p1, p2)]
    E, D, _ = oracle_model(ar, total, np.zeros(30), np.zeros(30), bulge, x, w).tabulate_delta(30)
    kw = dict(itermax=2, delta_table=(E, D), df2=halo)
    p64 = ctx.run_model(NR, NG, NPL, RMIN, RMAX, bulge, F.Rule(x, w), **kw)
    p32 = ctx.run_model(NR, NG, NPL, RMIN, RMAX, bulge, F.Rule(x, w, precision=A.FJ_PREC_MIXED), **kw)
    assert rel_rows(p32["coef6"][0], p64["coef6"][0]) < 1e-4
    assert rel_rows(p32["coef6_2"][0], p64["coef6_2"][0]) < 1e-4
    assert rel_rows(p32["phil"], p64["phil"]) < 1e-4


def test_two_component_arguments(ctx):
    bulge, halo = components()
    with pytest.raises(F.FJError, match="ncomp"):
        ctx.run_model(NR, NG, NPL, RMIN, RMAX, bulge, F.Rule(), itermax=1, df2=halo, twocomp_order=5)
