"""Restarting a model from its written coefficient file: k iterations, the file written
with 17 significant digits and read back, then m more iterations from its tables (and the
first run's focal-distance table, which the file does not hold) give the bits of one run
of k + m iterations.  From the reference's 6-digit file the restart lands within the
printed precision (relative 1e-4 per shell; the loop is contracting, so the rounding of
the restart point does not grow).  Both for one component and for the reference's
two-component order.  Restart tables of the wrong shape are argument errors.  Also the
external-potential mode, which adds a fixed potential to every iteration's."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402
from fjmodels_gb300 import _abi as A  # noqa: E402
from tests.helpers import rel_rows  # noqa: E402

pytestmark = pytest.mark.gpu

NR, NG, NPL, RMIN, RMAX = 40, 16, 5, 1e-2, 100.0


def _rule():
    return F.Rule(*F.tanh_sinh_rule(16), precision=A.FJ_PREC_MIXED)


def _write(path, out, digits, ng):
    mats = np.stack([out["coef6"][i] for i in (0, 1, 2, 3, 4, 5)] + [out["phil"], out["Pr"], out["Pr2"]])
    F.writeOut(str(path), out["ar"], mats, ng, (0.55, 0.55, 1.0, 1.0, 0.0, 1.0, 1.0, 1.667, 5.0), digits=digits)
    return F.readOut(str(path))


@pytest.mark.parametrize("two", [False, True])
def test_restart_from_written_tables(ctx, tmp_path, two):
    df = F.DFParams("Hernquist")
    kw = dict(df2=F.DFParams("NFW", mass=1.0, r0=10.0), twocomp_order=A.FJ_TWOCOMP_REFERENCE) if two else {}
    full = ctx.run_model(NR, NG, NPL, RMIN, RMAX, df, _rule(), itermax=3, **kw)
    part = ctx.run_model(NR, NG, NPL, RMIN, RMAX, df, _rule(), itermax=2, **kw)
    dt = (part["Egrid"], part["Dgrid"])
    r17 = _write(tmp_path / "m17.out", part, 17, NG)
    rest = ctx.run_model(NR, NG, NPL, 0, 0, df, _rule(), itermax=1, delta_table=dt, restart=r17, **kw)
    assert rest["iterations"] == 1
    for k in ("phil", "Pr", "Pr2", "coef6"):
        assert np.array_equal(rest[k], full[k]), k
    r6 = _write(tmp_path / "m6.out", part, 0, NG)
    rest6 = ctx.run_model(NR, NG, NPL, 0, 0, df, _rule(), itermax=1, delta_table=dt, restart=r6, **kw)
    assert rel_rows(rest6["phil"], full["phil"]) < 1e-4


def test_restart_arguments(ctx):
    df = F.DFParams("Hernquist")
    bad = {"ar": np.ones(NR), "phil": np.zeros((NR, NPL)), "Pr": np.zeros((NR, NPL)), "Pr2": np.zeros((NR, NPL - 1))}
    with pytest.raises(F.FJError):
        ctx.run_model(NR, NG, NPL, 0, 0, df, _rule(), itermax=1, restart=bad)
    bad["Pr2"] = np.zeros((NR, NPL))  # right shapes, but ar not increasing
    with pytest.raises(F.FJError):
        ctx.run_model(NR, NG, NPL, 0, 0, df, _rule(), itermax=1, restart=bad)


def test_external_potential_mode(ctx):
    """The reference's external mode (fJmodels.cpp:120-125, 134; the NFW halo of
    pot/models.cpp:61-65 with a = 25, GM = 0.01): the iterations start from guess + ext and
    every new potential is the model's own plus ext.  One iteration equals the explicit
    sequence Poisson(guess) + ext -> focal-distance table -> moments -> projection ->
    Poisson -> + ext, bit for bit."""
    rule = _rule()
    df = F.DFParams("Hernquist")
    ar = F.log_grid(RMIN, RMAX, NR)
    f64 = dict(dtype=torch.float64, device="cuda")
    d_ar = torch.tensor(ar, **f64)

    def poisson(rhl):
        t = [torch.zeros((NR, NPL), **f64) for _ in range(3)]
        ctx.computePhil(d_ar, torch.tensor(rhl, **f64), *t)
        return t

    ext = poisson(F.guess_rhl(ar, NG, NPL, "NFWext", mass=0.01, r0=25.0))
    ext_h = [t.cpu().numpy() for t in ext]
    out = ctx.run_model(NR, NG, NPL, RMIN, RMAX, df, rule, itermax=1, ext=ext_h)
    tot = [a + b for a, b in zip(poisson(F.guess_rhl(ar, NG, NPL, "Hernquist")), ext)]
    tot_h = [t.cpu().numpy() for t in tot]
    E, D, _ = F.tabulate_delta(ar, *tot_h)
    assert np.array_equal(out["Egrid"], E) and np.array_equal(out["Dgrid"], D)
    pot, delta = ctx.potential(d_ar, *tot), ctx.delta(torch.tensor(E, **f64), torch.tensor(D, **f64))
    new = [torch.zeros((NR, NPL), **f64) for _ in range(3)]
    grids, coef = torch.zeros((6, NR, NG), **f64), torch.zeros((6, NR, NPL), **f64)
    ctx.computeNewPhi(pot, delta, df, rule, NG, grids, coef, *new)
    torch.cuda.synchronize()
    for k, a, b in zip(("phil", "Pr", "Pr2"), new, ext):
        assert np.array_equal(out[k], (a + b).cpu().numpy()), k
    with pytest.raises(F.FJError):
        ctx.run_model(NR, NG, NPL, RMIN, RMAX, df, rule, itermax=1, ext=[e[:-1] for e in ext_h])
