"""Anderson mixing of the self-consistent loop (fj_anderson_step; fj_run_model's accel).

The reference iterates the plain map (fJmodels.cpp:131-143).  The mixed loop must
reach the same fixed point, in fewer iterations, stopping by the same test (the
change one plain step makes is below tol), and end with a plain step.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402
from fjmodels_gb300 import _abi as A  # noqa: E402

pytestmark = pytest.mark.gpu


def _tables(nr=16, npl=3, seed=1):
    g = np.random.default_rng(seed)
    xs = g.uniform(-1.0, 1.0, (3, nr, npl))
    xs[0, :, 0] = -1.0 - g.uniform(0, 1, nr)  # the potential's monopole: the stopping test's scale
    return xs


def test_anderson_linear_map(ctx):
    """On a linear contraction with two rates (0.3 and 0.6 by multipole) depth 2 finds the
    fixed point to rounding in a few steps; the plain map would still be ~5 % away."""
    nr, npl = 16, 3
    xs = torch.tensor(_tables(nr, npl), dtype=torch.float64, device="cuda")
    rate = torch.full((3, nr, npl), 0.6, dtype=torch.float64, device="cuda")
    rate[:, :, 1:] = 0.3
    x = torch.zeros_like(xs)
    x[0, :, 0] = -1.0
    ctx.anderson_reset(2)
    changes = []
    for _ in range(10):
        g = (xs + rate * (x - xs)).contiguous()
        changes.append(ctx.anderson_step(x, g))
    assert changes[-1] < 1e-12, changes
    assert changes[0] > 0.1
    assert float((x - xs).abs().max()) < 1e-12
    # the first step has no history: x = g exactly
    x = torch.zeros_like(xs)
    x[0, :, 0] = -1.0
    ctx.anderson_reset(2)
    g = (xs + rate * (x - xs)).contiguous()
    ctx.anderson_step(x, g)
    assert torch.equal(x, g)
    # mixing factor 1.6: the same fixed point (host reference of the same step: 1e-15 by the 8th)
    x = torch.zeros_like(xs)
    x[0, :, 0] = -1.0
    ctx.anderson_reset(2, 1.6)
    x0 = x.clone()
    g = (xs + rate * (x - xs)).contiguous()
    ctx.anderson_step(x, g)
    assert torch.allclose(x, x0 + 1.6 * (g - x0), rtol=0, atol=1e-15)  # no history: x + beta (g - x)
    for _ in range(9):
        g = (xs + rate * (x - xs)).contiguous()
        ch = ctx.anderson_step(x, g)
    assert ch < 1e-12 and float((x - xs).abs().max()) < 1e-12


def test_anderson_restarts_when_diverging(ctx):
    """A change that grows by more than a factor 2 drops the history: that step is plain."""
    nr, npl = 12, 2
    xs = torch.tensor(_tables(nr, npl, seed=3), dtype=torch.float64, device="cuda")
    x = xs.clone()
    x[0] += 1e-3
    ctx.anderson_reset(2)
    for _ in range(3):
        g = (xs + 0.5 * (x - xs)).contiguous()
        ctx.anderson_step(x, g)
    g = (x + 1.0).contiguous()  # a change far larger than the last
    g[0, :, 0] = x[0, :, 0] - 0.5
    ch = ctx.anderson_step(x, g)
    assert ch > 0.1 and torch.equal(x, g)


def test_anderson_arguments(ctx):
    with pytest.raises(F.FJError):
        ctx.anderson_reset(A.FJ_ANDERSON_MAX_DEPTH + 1)
    with pytest.raises(F.FJError):
        ctx.anderson_reset(-1)
    for beta in (0.0, -1.0, 4.5):
        with pytest.raises(F.FJError):
            ctx.anderson_reset(2, beta)
    x = torch.zeros((3, 4, 2), dtype=torch.float64, device="cuda")
    with pytest.raises(F.FJError):
        ctx.anderson_step(x, torch.zeros((3, 4, 3), dtype=torch.float64, device="cuda"))


@pytest.fixture
def cumulative(ctx):
    ctx.set_poisson(A.FJ_POISSON_CUMULATIVE)
    yield ctx
    ctx.set_poisson(A.FJ_POISSON_QAGS)


def test_run_model_accel_reaches_the_fixed_point(cumulative):
    """A small Hernquist model (24 x 8, l <= 6, the reference's live velocity rule) in the
    mixed form: the plain loop and the depth-2 mixed loop to tol = 1e-5, and the plain loop
    run on to its floor (the fixed point).  The mixed loop takes fewer iterations and its
    converged potential and density multipoles are at least as close to the fixed point as
    the plain loop's (up to 20 %), each within 1e-4 of it."""
    ctx = cumulative
    df = F.DFParams("Hernquist")
    rule = F.Rule(F.XPT11, F.XW11, precision=A.FJ_PREC_MIXED)
    args = (24, 8, 4, 0.01, 100.0, df, rule)
    plain = ctx.run_model(*args, itermax=60, tol=1e-5)
    mixed = ctx.run_model(*args, itermax=60, tol=1e-5, accel=2)
    truth = ctx.run_model(*args, itermax=45, tol=0.0)
    assert plain["last_change"] < 1e-5 and mixed["last_change"] < 1e-5
    assert mixed["iterations"] < plain["iterations"], (mixed["iterations"], plain["iterations"])

    def dist(r):
        s = np.abs(truth["phil"][:, :1])
        dphi = np.max(np.abs(r["phil"] - truth["phil"]) / s)
        rho = truth["coef6"][0]
        drho = np.max(np.abs(r["coef6"][0] - rho) / np.abs(rho[:, :1]))
        return dphi, drho

    (pp, pr), (mp, mr) = dist(plain), dist(mixed)
    print(f"iterations plain {plain['iterations']} mixed {mixed['iterations']}; vs the fixed point: "
          f"plain phil {pp:.2e} rho {pr:.2e}, mixed phil {mp:.2e} rho {mr:.2e}")
    assert mp < 1e-4 and mr < 1e-4
    assert mp <= 1.2 * pp + 1e-9 and mr <= 1.2 * pr + 1e-9
    # the bench's setting: mixing factor 1.6
    relaxed = ctx.run_model(*args, itermax=60, tol=1e-5, accel=2, accel_beta=1.6)
    rp, rr = dist(relaxed)
    print(f"mixed, beta 1.6: {relaxed['iterations']} iterations, phil {rp:.2e} rho {rr:.2e}")
    assert relaxed["last_change"] < 1e-5 and relaxed["iterations"] < plain["iterations"]
    assert rp <= 1.2 * pp + 1e-9 and rr <= 1.2 * pr + 1e-9


def test_run_model_accel_range(ctx):
    """A depth outside [0, FJ_ANDERSON_MAX_DEPTH] is an argument error."""
    df = F.DFParams("Hernquist")
    rule = F.Rule(F.XPT11, F.XW11, precision=A.FJ_PREC_MIXED)
    with pytest.raises(F.FJError, match="accel"):
        ctx.run_model(24, 8, 4, 0.01, 100.0, df, rule, itermax=2, accel=A.FJ_ANDERSON_MAX_DEPTH + 1)
    with pytest.raises(F.FJError, match="accel_beta"):
        ctx.run_model(24, 8, 4, 0.01, 100.0, df, rule, itermax=2, accel=2, accel_beta=5.0)
