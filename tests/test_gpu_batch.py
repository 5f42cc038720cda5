"""Many models in one launch (fj_moments_batch) and iterated together with the
per-iteration sequence replayed as a CUDA graph (fj_run_model_batch): the
batched results are those of the one-model calls, bit for bit, in both forms.
Three small models of different grid sizes, multipole orders, profiles and
DFs, a 10-point tanh-sinh velocity rule."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402
from fjmodels_gb300 import _abi as A  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

MODELS = [
    dict(nr=16, ngauss=6, npoly=3, rmin=0.01, rmax=100.0, df=F.DFParams("Hernquist", 0.6, 0.9, 1.0, 1.0)),
    dict(nr=24, ngauss=8, npoly=5, rmin=0.005, rmax=300.0, df=F.DFParams("NFW", 0.55, 0.55, 1.0, 1.0, chi=1.0, k=0.5)),
    dict(nr=20, ngauss=4, npoly=4, rmin=0.02, rmax=50.0, df=F.DFParams("Isochrone", 0.8, 0.4, 1.0, 1.0, chi=0.5)),
]


def dev(a):
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def setup(m):
    ar = F.log_grid(m["rmin"], m["rmax"], m["nr"])
    phil, Pr, Pr2 = O.compute_phil(ar, F.guess_rhl(ar, m["ngauss"], m["npoly"], m["df"].model))
    E, D, _ = F.tabulate_delta(ar, phil, Pr, Pr2)
    return [dev(t) for t in (ar, phil, Pr, Pr2)], (dev(E), dev(D))


@pytest.mark.parametrize("precision", [A.FJ_PREC_FP64, A.FJ_PREC_MIXED])
def test_moments_batch_equals_single(ctx, precision):
    rule = F.Rule(*F.tanh_sinh_rule(10), precision=precision)
    items, singles = [], []
    for m in MODELS:
        tabs, (E, D) = setup(m)
        pot, delta = ctx.potential(*tabs), ctx.delta(E, D)
        g1 = torch.zeros((6, m["nr"], m["ngauss"]), dtype=torch.float64, device="cuda")
        ctx.moments(pot, delta, m["df"], rule, m["ngauss"], g1)
        singles.append(g1)
        gb = torch.zeros_like(g1)
        items.append((pot, delta, m["df"], m["ngauss"], gb))
    st = ctx.moments_batch(items, rule)
    assert st.nodes == sum(m["nr"] * m["ngauss"] for m in MODELS) * 10 ** 3
    for (_, _, _, _, gb), g1 in zip(items, singles):
        torch.cuda.synchronize()
        assert torch.equal(gb, g1)


@pytest.mark.parametrize("use_graph", [False, True])
def test_run_model_batch_equals_single(ctx, use_graph):
    rule = F.Rule(*F.tanh_sinh_rule(10))
    outs = ctx.run_model_batch(MODELS, rule, itermax=3, use_graph=use_graph)
    for m, ob in zip(MODELS, outs):
        o1 = ctx.run_model(m["nr"], m["ngauss"], m["npoly"], m["rmin"], m["rmax"], m["df"], rule, itermax=3)
        assert ob["iterations"] == 3
        for key in ("coef6", "phil", "Pr", "Pr2", "Egrid", "Dgrid"):
            np.testing.assert_array_equal(ob[key], o1[key], err_msg=key)
        np.testing.assert_array_equal(ob["vir7"], o1["vir7"])


def test_run_model_batch_mixed_graph(ctx):
    rule = F.Rule(*F.tanh_sinh_rule(10), precision=A.FJ_PREC_MIXED)
    outs = ctx.run_model_batch(MODELS, rule, itermax=2, use_graph=True)
    for m, ob in zip(MODELS, outs):
        o1 = ctx.run_model(m["nr"], m["ngauss"], m["npoly"], m["rmin"], m["rmax"], m["df"], rule, itermax=2)
        np.testing.assert_array_equal(ob["phil"], o1["phil"])


def test_batch_arguments(ctx):
    rule = F.Rule(*F.tanh_sinh_rule(10))
    other = F.Rule(*F.tanh_sinh_rule(12))
    with pytest.raises(F.FJError, match="velocity rule"):
        bad = [dict(MODELS[0]), dict(MODELS[1], rule=other)]
        # a second model with another rule: the C entry point checks every config's rule
        import ctypes as C
        n = 2
        cfgs = (A.fj_model_config * n)()
        ress = (A.fj_model_result * n)()
        bufs = []
        for i, (m, r) in enumerate(zip(bad, (rule, other))):
            nr, npl = m["nr"], m["npoly"]
            b = [np.zeros(nr), np.zeros(6 * nr * npl), np.zeros(nr * npl), np.zeros(nr * npl), np.zeros(nr * npl),
                 np.zeros(30), np.zeros(30)]
            bufs.append(b)
            cfgs[i] = A.fj_model_config(nr, m["ngauss"], npl, 30, m["rmin"], m["rmax"], 0, 1.0, 1.0, 1.0, m["df"].c,
                                        r.c, 1, 0.0, None, None)
            ress[i] = A.fj_model_result(*[b_.ctypes.data_as(A.DP) for b_ in b], None)
        ctx._check(ctx.lib.fj_run_model_batch(ctx.h, n, cfgs, ress, 0), "fj_run_model_batch")


def test_run_model_batch_mixes_component_counts(ctx):
    """One- and two-component models (summed order) in one batch: each gives the bits of its
    own fj_run_model, component 2's coefficients and virial sums included."""
    rule = F.Rule(*F.tanh_sinh_rule(10), precision=A.FJ_PREC_MIXED)
    halo = F.DFParams("NFW", dphi_h=0.5, dz_h=0.8, dphi_g=1.0, dz_g=1.2, mass=1.0, r0=10.0)
    models = [MODELS[0], dict(MODELS[1], df=F.DFParams("Hernquist", mass=0.1, r0=1.0), df2=halo)]
    for use_graph in (False, True):
        outs = ctx.run_model_batch(models, rule, itermax=2, use_graph=use_graph)
        for m, ob in zip(models, outs):
            kw = dict(df2=m["df2"], twocomp_order=A.FJ_TWOCOMP_SUMMED) if "df2" in m else {}
            o1 = ctx.run_model(m["nr"], m["ngauss"], m["npoly"], m["rmin"], m["rmax"], m["df"], rule, itermax=2, **kw)
            for key in ("phil", "Pr", "Pr2", "coef6", "vir7") + (("coef6_2", "vir7_2") if kw else ()):
                np.testing.assert_array_equal(ob[key], o1[key], err_msg=f"{key} graph={use_graph}")
