"""The mixed-precision phase-space form (FJ_PREC_MIXED) against the FP64 plain
form, the CPU oracle and the reference's own outputs.

The mixed form computes the turning points, the QAGS momentum integrals and the
DF in FP32 (turning points at the u/v limits and all accumulation in FP64), so
it is not bit-faithful to the reference; its gate is the density error of the
self-consistent loop: relative 1e-4 on rho at every grid point and on the
density multipoles (scaled by the monopole of the shell), and 1e-4 on the
dispersions.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402
from fjmodels_gb300 import _abi as A  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.conftest import load_golden  # noqa: E402
from tests.helpers import oracle_model, rel, rel_rows  # noqa: E402

pytestmark = pytest.mark.gpu
MIXED_TOL = 1e-4


def dev(a):
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def df_of(meta):
    p = meta["p"]
    return F.DFParams(p["model"], p["dphi_h"], p["dz_h"], p["dphi_g"], p["dz_g"], p["chi"], p["mass"], p["r0"],
                      k=meta["k"], kind=1 if meta["df"] == "qiso" else 0)


def mixed_rule(x=F.XPT11, w=F.XW11):
    return F.Rule(x, w, precision=A.FJ_PREC_MIXED)


@pytest.mark.parametrize("name", ["hern_dpl", "nfw_dpl_rot"])
def test_mixed_compute_new_phi_vs_reference(ctx, name):
    """computeNewPhi (pot/potLeg.cpp:76-82) in the mixed form vs the reference's first iteration."""
    g, meta, _ = load_golden(name)
    nr, ng, npl = meta["nr"], meta["ng"], meta["np"]
    ar = dev(g["ar"])
    tabs = [dev(g[k].reshape(nr, npl)) for k in ("guess_phil", "guess_Pr", "guess_Pr2")]
    pot = ctx.potential(ar, *tabs)
    delta = ctx.delta(dev(g["Egrid"]), dev(g["Dgrid"]))
    grids = torch.zeros((6, nr, ng), dtype=torch.float64, device="cuda")
    coef = torch.zeros((6, nr, npl), dtype=torch.float64, device="cuda")
    outs = [torch.zeros((nr, npl), dtype=torch.float64, device="cuda") for _ in range(3)]
    st = ctx.computeNewPhi(pot, delta, df_of(meta), mixed_rule(), ng, grids, coef, *outs)
    assert st.nodes == nr * ng * 22 ** 3 and 0 <= st.escalated <= st.bound
    c = host(coef)
    for q, key in ((0, "rhl"), (2, "sigRl"), (3, "sigpl"), (4, "sigzl")):
        assert rel_rows(c[q], g["it0_" + key].reshape(nr, npl)) < MIXED_TOL, key
    for o, key in zip(outs, ("it0_phil", "it0_Pr")):
        assert rel_rows(host(o), g[key].reshape(nr, npl)) < MIXED_TOL, key


def _nfw_80(rule_xw):
    """The 80-radius NFW potential (0.001..300, l <= 12) of the guess density, a spread
    of 48 meridional points (every 7th radius x 4 polar angles incl. the near-equatorial
    and near-polar nodes) and the DF of the rotating NFW model (chi = 1, k = 0.5)."""
    nr, ng, npl = 80, 40, 7
    ar = F.log_grid(1e-3, 300.0, nr)
    rhl = F.guess_rhl(ar, ng, npl, "NFW")
    phil, Pr, Pr2 = O.compute_phil(ar, rhl)
    E, D, _ = F.tabulate_delta(ar, phil, Pr, Pr2)
    ci, _ = F.gauleg(0, 1, ng)
    ci = np.sort(ci)
    M = np.array([[ar[n] * np.sqrt(1 - ci[k] ** 2), ar[n] * ci[k]] for n in range(0, nr, 7)
                  for k in (0, ng // 3, 2 * ng // 3, ng - 1)])
    df = F.DFParams("NFW", chi=1.0, k=0.5)
    return (ar, phil, Pr, Pr2, E, D), M, df


@pytest.mark.parametrize("rule", ["xpt11", "tanh22"])
def test_mixed_vs_plain_nfw_80(ctx, rule):
    """Mixed vs plain FP64 on the 80-radius rotating NFW workload, both velocity rules."""
    x, w = (F.XPT11, F.XW11) if rule == "xpt11" else F.tanh_sinh_rule(22)
    (ar, phil, Pr, Pr2, E, D), M, df = _nfw_80(None)
    pot = ctx.potential(dev(ar), dev(phil), dev(Pr), dev(Pr2))
    delta = ctx.delta(dev(E), dev(D))
    out64 = torch.zeros((6, len(M)), dtype=torch.float64, device="cuda")
    out32 = torch.zeros((6, len(M)), dtype=torch.float64, device="cuda")
    ctx.moments_points(pot, delta, df, F.Rule(x, w), dev(M), out64)
    st = ctx.moments_points(pot, delta, df, F.Rule(x, w, precision=A.FJ_PREC_MIXED), dev(M), out32)
    a, b = host(out32).T, host(out64).T
    assert rel(a[:, 0], b[:, 0]) < MIXED_TOL
    assert rel(a[:, [2, 3, 4]], b[:, [2, 3, 4]]) < MIXED_TOL
    # vrot is a nearly cancelling sum: compare on the scale of the dispersion
    assert np.max(np.abs(a[:, 1] - b[:, 1]) / b[:, 3]) < MIXED_TOL
    # escalated turning points are rare; a node whose FP32 solve hits a cap is solved again
    # by the FP64 pass, so no failure remains (the plain form has none on this workload)
    assert st.escalated < 0.01 * st.bound and st.failures == 0
    assert st.fail_quad == st.fail_bracket == st.fail_root == 0
    assert 0 <= st.resolved64 < 0.01 * st.bound
    # the deferred FP64 pass adds to fixed per-block sums in slot order: the same bits again
    out2 = torch.zeros_like(out32)
    st2 = ctx.moments_points(pot, delta, df, F.Rule(x, w, precision=A.FJ_PREC_MIXED), dev(M), out2)
    assert torch.equal(out2, out32) and st2.resolved64 == st.resolved64


def test_mixed_vs_oracle_nfw_80(ctx):
    """Mixed form vs the CPU oracle (the reference's algorithm in FP64) on six points of
    the 80-radius workload: the innermost shell, mid radii on the equator and the pole,
    the outermost shell."""
    (ar, phil, Pr, Pr2, E, D), M, df = _nfw_80(None)
    pick = [0, 3, 13, 22, 30, 47]
    M = M[pick]
    pot = ctx.potential(dev(ar), dev(phil), dev(Pr), dev(Pr2))
    delta = ctx.delta(dev(E), dev(D))
    out = torch.zeros((6, len(M)), dtype=torch.float64, device="cuda")
    ctx.moments_points(pot, delta, df, mixed_rule(), dev(M), out)
    m = O.Model(ar, phil, Pr, Pr2, E, D, 40, alpha=1.667, beta=3.0, chi=1.0, k=0.5)
    ref = np.array([m.rhofDF(R, z)[0] for R, z in M])
    got = host(out).T
    assert rel(got[:, [0, 2, 3, 4]], ref[:, [0, 2, 3, 4]]) < MIXED_TOL


@pytest.fixture
def cumulative(ctx):
    """The loop comparisons run with the cumulative Poisson solve, as the chosen form does:
    with the adaptive one, a density difference of 1e-6 between the forms can flip one of
    its subdivision decisions and move the next potential by up to ~1e-3."""
    ctx.set_poisson(A.FJ_POISSON_CUMULATIVE)
    yield ctx
    ctx.set_poisson(A.FJ_POISSON_QAGS)


def test_mixed_run_model_vs_plain(cumulative):
    """Two iterations of the whole loop in both forms: density multipoles and the
    virial ratio within the mixed gate.  On the Hernquist fixture: on the 12 x 4 NFW
    fixture one grid point (r ~ 46, cos theta ~ 0.67, three times the density of its
    neighbours) is decided by a single node, and the reference's own FP64 algorithm
    moves it by 1.3 % between potentials that differ by 3e-7, so a second iteration
    there compares that discontinuity, not the two forms."""
    ctx = cumulative
    g, meta, _ = load_golden("hern_dpl")
    nr, ng, npl = meta["nr"], meta["ng"], meta["np"]
    df = df_of(meta)
    dt = (g["Egrid"], g["Dgrid"])
    p64 = ctx.run_model(nr, ng, npl, meta["rmin"], meta["rmax"], df, F.Rule(), itermax=2, delta_table=dt)
    p32 = ctx.run_model(nr, ng, npl, meta["rmin"], meta["rmax"], df, mixed_rule(), itermax=2, delta_table=dt)
    assert p32["iterations"] == 2
    assert rel_rows(p32["coef6"][0], p64["coef6"][0]) < MIXED_TOL
    assert rel_rows(p32["phil"], p64["phil"]) < MIXED_TOL
    v64, v32 = p64["vir7"], p32["vir7"]
    assert abs(v32[4] / (v32[0] + v32[1]) - v64[4] / (v64[0] + v64[1])) < 1e-4


def test_mixed_rejects_unsupported(ctx):
    """The mixed form takes the double-power-law DF with QAGS momentum integrals only;
    anything else is an argument error, not a silent switch to another form."""
    g, meta, _ = load_golden("hern_qiso")
    nr, npl = meta["nr"], meta["np"]
    ar = dev(g["ar"])
    tabs = [dev(g[k].reshape(nr, npl)) for k in ("guess_phil", "guess_Pr", "guess_Pr2")]
    pot = ctx.potential(ar, *tabs)
    delta = ctx.delta(dev(g["Egrid"]), dev(g["Dgrid"]))
    M = dev([[1.0, 0.5]])
    out = torch.zeros((6, 1), dtype=torch.float64, device="cuda")
    with pytest.raises(F.FJError, match="mixed form"):
        ctx.moments_points(pot, delta, df_of(meta), mixed_rule(), M, out)
    with pytest.raises(F.FJError, match="mixed form"):
        ctx.moments_points(pot, delta, F.DFParams("Hernquist"), F.Rule(jquad=8, precision=A.FJ_PREC_MIXED), M, out)
    with pytest.raises(F.FJError, match="precision"):
        ctx.moments_points(pot, delta, F.DFParams("Hernquist"), F.Rule(precision=7), M, out)


def test_mixed_configurations_agree(ctx):
    """Every build and node range of the mixed kernel gives the same moments: within one
    form (static shares of the node list: variants 0-3; nodes taken as lanes free up:
    4-7) up to the summation order of the per-thread sums (relative 1e-12), and the two
    forms give the same bits for the same node range (the dynamic form sums the same terms
    in the same order after the solves).  The autotuner keeps one of them, and
    out-of-range settings are argument errors."""
    (ar, phil, Pr, Pr2, E, D), M, df = _nfw_80(None)
    pot = ctx.potential(dev(ar), dev(phil), dev(Pr), dev(Pr2))
    delta = ctx.delta(dev(E), dev(D))
    rule = F.Rule(*F.tanh_sinh_rule(22), precision=A.FJ_PREC_MIXED)
    Mt = dev(M[::3])
    saved = ctx.mixed_config()
    outs = {}
    try:
        for v in range(8):
            for c in (128, 2048, 8192):
                ctx.set_mixed_config(v, c)
                out = torch.zeros((6, Mt.shape[0]), dtype=torch.float64, device="cuda")
                ctx.moments_points(pot, delta, df, rule, Mt, out)
                outs[v, c] = host(out)
        for (v, c), o in outs.items():
            first = outs[(v // 4) * 4, 128]
            assert rel(o[[0, 2, 3, 4]], first[[0, 2, 3, 4]]) < 1e-12, (v, c)
        for c in (128, 2048, 8192):
            for v in range(4):
                assert np.array_equal(outs[v + 4, c], outs[v, c]), (v, c)
        v, c, ms = ctx.autotune_mixed(pot, delta, df, rule, Mt)
        assert 0 <= v < 8 and c in (1024, 2048, 4096) and ms > 0
        for bad in ((8, 2048), (0, 64), (0, 8193)):
            with pytest.raises(F.FJError, match="set_mixed_config"):
                ctx.set_mixed_config(*bad)
    finally:
        ctx.set_mixed_config(*saved)


def test_mixed_loop_vs_plain_c1(cumulative):
    """The whole self-consistent loop of the 40 x 20 Hernquist configuration (l <= 8, the
    reference's live velocity rule, 5 iterations from the analytic guess) in the chosen
    form against the plain FP64 form: density multipoles and potential within 1e-4 of
    the FP64 ones (relative to each shell's monopole) and the virial ratio within 1e-4,
    after the iterations have compounded the per-iteration differences."""
    ctx = cumulative
    df = F.DFParams("Hernquist")
    args = (40, 20, 5, 0.01, 100.0, df)
    p64 = ctx.run_model(*args, F.Rule(), itermax=5)
    p32 = ctx.run_model(*args, mixed_rule(), itermax=5, delta_table=(p64["Egrid"], p64["Dgrid"]))
    d_rho = rel_rows(p32["coef6"][0], p64["coef6"][0])
    d_phi = rel_rows(p32["phil"], p64["phil"])
    v64, v32 = p64["vir7"], p32["vir7"]
    d_vir = abs(v32[4] / (v32[0] + v32[1]) - v64[4] / (v64[0] + v64[1]))
    print(f"C1 after 5 iterations: rho multipoles {d_rho:.2e}, potential {d_phi:.2e}, virial ratio {d_vir:.2e}; "
          f"wall {p64['wall_ms'] / 1e3:.1f} s (FP64) vs {p32['wall_ms'] / 1e3:.2f} s (mixed)")
    assert d_rho < 1e-4 and d_phi < 1e-4 and d_vir < 1e-4
