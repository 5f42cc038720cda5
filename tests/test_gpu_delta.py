"""The focal-distance table on the GPU (fj_tabulate_delta_batch: the host's
tabulateDelta code, delta/tabulate.cpp:13-38 and delta/Delta.cpp, one thread per
(model, energy), 8 per block).  The focal-distance fit is not continuous in rounding (one unit in
the last place of the orbit equations moves entries by tens of per cent; the host code
does the same), so the GPU table is checked for what is stable: the energies against
the host's and the reference's to 1e-12, every focal distance within the spread the fit
itself shows under one-ulp perturbations, run-to-run identity, and the density moments a
table gives -- within a few per cent of the host table's (the Staeckel fudge depends on
the focal distance only through the quality of its fit; 2.6e-2 measured on the GB300,
bound 5e-2).  In the model loops: a GPU table gives
the same bits in fj_run_model and fj_run_model_batch (graph or not), and re-tabulating
after every iteration uses the table of the potential the previous iteration produced."""
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402
from fjmodels_gb300 import _abi as A  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.conftest import load_golden  # noqa: E402
from tests.helpers import rel  # noqa: E402

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def _models(n, seed):
    """C4-like models: type, grid and sizes drawn from a seeded generator."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        model = ["Hernquist", "Isochrone", "NFW"][rng.integers(3)]
        nr, npl = int(rng.choice([32, 48, 64])), 5
        ar = F.log_grid(1e-2, 100.0 if model != "NFW" else 300.0, nr)
        rhl = F.guess_rhl(ar, 16, npl, model)
        out.append((ar, *O.compute_phil(ar, rhl)))
    return out


def test_gpu_table_against_host_table(ctx):
    tabs = _models(24, 5)
    pots = [ctx.potential(*[dev(t) for t in tb]) for tb in tabs]
    t0 = time.perf_counter()
    E, D, status = ctx.tabulate_delta_batch(pots, 30)
    torch.cuda.synchronize()
    t_gpu = time.perf_counter() - t0
    E2, D2, _ = ctx.tabulate_delta_batch(pots, 30)
    assert torch.equal(E, E2) and torch.equal(D, D2)  # run to run
    E, D = E.cpu().numpy(), D.cpu().numpy()
    t0 = time.perf_counter()
    host = [F.tabulate_delta(*tb) for tb in tabs]
    t_host = time.perf_counter() - t0
    dev_rel = [float(np.median(np.abs(D[m] - Dh) / np.abs(Dh))) for m, (_, Dh, _) in enumerate(host)]
    print(f"24 models: GPU {t_gpu * 1e3:.0f} ms, host (one thread) {t_host * 1e3:.0f} ms; "
          f"median |dD2/D2| per model: {np.round(dev_rel, 3)}")
    for m, (Eh, Dh, rc) in enumerate(host):
        assert rel(E[m], Eh) < 1e-12, m
        assert np.all(np.isfinite(D[m])), m
    # the densities the tables give, on a spread of points of the first NFW model
    m = next(i for i, tb in enumerate(tabs) if tb[0][-1] > 200)
    ar, phil, Pr, Pr2 = tabs[m]
    pts = np.array([[r * np.sqrt(1 - c * c), r * c] for r in ar[::6] for c in (0.1, 0.5, 0.9)])
    rule = F.Rule(*F.tanh_sinh_rule(16), precision=A.FJ_PREC_MIXED)
    df = F.DFParams("NFW", chi=1.0, k=0.5)
    rho = []
    for Et, Dt in ((E[m], D[m]), host[m][:2]):
        out = torch.zeros((6, len(pts)), dtype=torch.float64, device="cuda")
        ctx.moments_points(pots[m], ctx.delta(dev(Et), dev(Dt)), df, rule, dev(pts), out)
        rho.append(out[0].cpu().numpy())
    drho = np.max(np.abs(rho[0] - rho[1]) / rho[1])
    print(f"densities with the GPU table vs the host table: max rel difference {drho:.2e}")
    assert drho < 5e-2


@pytest.mark.parametrize("name", ["hern_dpl", "nfw_dpl_rot", "c1_hern", "twocomp_ref"])
def test_gpu_table_entrywise_against_reference(ctx, name):
    """The GPU table against the reference's own (the fixture's, which the host code
    reproduces bit for bit), entry by entry.  The fit is chaotic in rounding, so the bound
    is the fit's own spread: the host tables of the same potential with its multipoles
    scaled by 1 + j 2^-52, j = -16..16, give each entry an envelope [lo, hi]; each GPU
    entry must lie within it widened by half its width on each side, and at least 90 % of
    them inside it (measured: 115 of 120 inside, the rest within 0.34 widths).  The
    energies agree to 1e-12."""
    g, meta, _ = load_golden(name)
    nr, npl = meta["nr"], meta["np"]
    tabs = [g[k].reshape(nr, npl) for k in ("guess_phil", "guess_Pr", "guess_Pr2")]
    pot = ctx.potential(dev(g["ar"]), *[dev(t) for t in tabs])
    E, D, _ = ctx.tabulate_delta_batch([pot], 30)
    E, D = E.cpu().numpy()[0], D.cpu().numpy()[0]
    assert rel(E, g["Egrid"]) < 1e-12
    host = np.array([F.tabulate_delta(g["ar"], tabs[0] * (1 + j * 2.0 ** -52), tabs[1], tabs[2])[1]
                     for j in range(-16, 17)])
    assert np.array_equal(host[16], g["Dgrid"])  # the unperturbed host table is the reference's
    lo, hi = host.min(0), host.max(0)
    w = hi - lo
    inside = (D >= lo) & (D <= hi)
    print(f"{name}: {inside.sum()}/30 GPU entries inside the host envelope; median |dD2/D2| against the "
          f"reference {np.median(np.abs(D - g['Dgrid']) / np.abs(g['Dgrid'])):.3f}")
    assert np.all((D >= lo - w / 2) & (D <= hi + w / 2))
    assert inside.sum() >= 27


MODELS = [dict(nr=32, ngauss=12, npoly=4, rmin=1e-2, rmax=100.0, df=F.DFParams("Hernquist")),
          dict(nr=40, ngauss=16, npoly=5, rmin=1e-2, rmax=300.0, df=F.DFParams("NFW", chi=1.0, k=0.5))]


@pytest.mark.parametrize("use_graph", [False, True])
def test_gpu_tables_in_the_model_loops(ctx, use_graph):
    rule = F.Rule(*F.tanh_sinh_rule(10), precision=A.FJ_PREC_MIXED)
    for every in (0, 1):
        outs = ctx.run_model_batch(MODELS, rule, itermax=3, use_graph=use_graph, delta_gpu=True, delta_every=every)
        for m, ob in zip(MODELS, outs):
            o1 = ctx.run_model(m["nr"], m["ngauss"], m["npoly"], m["rmin"], m["rmax"], m["df"], rule, itermax=3,
                               delta_gpu=True, delta_every=every)
            for key in ("phil", "Pr", "Pr2", "coef6", "Egrid", "Dgrid"):
                np.testing.assert_array_equal(ob[key], o1[key], err_msg=f"{key} every={every}")


def test_retabulated_table_is_the_previous_potentials(ctx):
    m = MODELS[1]
    rule = F.Rule(*F.tanh_sinh_rule(10), precision=A.FJ_PREC_MIXED)
    args = (m["nr"], m["ngauss"], m["npoly"], m["rmin"], m["rmax"], m["df"], rule)
    one = ctx.run_model(*args, itermax=1, delta_gpu=True)
    two = ctx.run_model(*args, itermax=2, delta_gpu=True, delta_every=1)
    pot = ctx.potential(dev(one["ar"]), dev(one["phil"]), dev(one["Pr"]), dev(one["Pr2"]))
    E, D, _ = ctx.tabulate_delta_batch([pot], 30)
    np.testing.assert_array_equal(two["Egrid"], E.cpu().numpy()[0])
    np.testing.assert_array_equal(two["Dgrid"], D.cpu().numpy()[0])
    assert not np.array_equal(two["Dgrid"], one["Dgrid"])
    with pytest.raises(F.FJError):
        ctx.run_model_batch(MODELS, rule, itermax=2, delta_gpu=False, delta_every=1)
