"""Parity of the CUDA path (called through the C ABI) with the reference's own
outputs (golden fixtures) and with the CPU oracle.

Tolerances: FP64 plain form, relative 1e-9 on the density and potential
multipole coefficients (scaled by the monopole of the same radius), 1e-9 on
actions and point moments, 1e-6 on the virial ratios.  vrot is a difference
of nearly cancelling sums (the reference's 1e-6 velocity offset makes it
nonzero for a non-rotating model) and is compared against the scale of the
second moments instead.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.conftest import load_golden  # noqa: E402
from tests.helpers import oracle_model, rel, rel_rows  # noqa: E402

pytestmark = pytest.mark.gpu
SCENARIOS = ["hern_dpl", "nfw_dpl_rot", "hern_qiso"]
TOL = 1e-9


def rel_shells(a, ref):
    """|a-ref| over (|monopole of the shell| + 1e-10 |central monopole|): the 1e-9 gate on
    multipole coefficients, with a floor for the two outermost shells, whose density is
    1e-11..1e-10 of the centre; there, after two iterations, the reference's own builds with
    and without FMA contraction differ by 1.6e-9 in the per-shell measure, and the GPU
    (whose exp/log/pow round differently from the host's libm) by 1.4e-9."""
    ref = np.asarray(ref)
    a = np.asarray(a).reshape(ref.shape)
    scale = np.abs(ref[:, :1]) + 1e-10 * np.abs(ref[0, 0])
    r = np.abs(a - ref) / scale
    i = np.unravel_index(np.argmax(r), r.shape)
    print(f"rel_shells max {r[i]:.3e} at shell {i[0]} coefficient {i[1]}: {a[i]!r} vs {ref[i]!r}")
    return float(r[i])


def dev(a):
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def df_of(meta):
    p = meta["p"]
    return F.DFParams(p["model"], p["dphi_h"], p["dz_h"], p["dphi_g"], p["dz_g"], p["chi"], p["mass"], p["r0"],
                      k=meta["k"], kind=1 if meta["df"] == "qiso" else 0)


def guess_pot(ctx, g, meta):
    nr, npl = meta["nr"], meta["np"]
    ar = dev(g["ar"])
    tabs = [dev(g[k].reshape(nr, npl)) for k in ("guess_phil", "guess_Pr", "guess_Pr2")]
    return ar, tabs, ctx.potential(ar, *tabs)


@pytest.mark.parametrize("name", SCENARIOS)
def test_potential_eval(ctx, name):
    g, meta, pts = load_golden(name)
    ar, tabs, pot = guess_pot(ctx, g, meta)
    P = np.array([[float(a[1]), float(a[2])] for a in pts if a[0] == "P"])
    out = torch.zeros((len(P), 3), dtype=torch.float64, device="cuda")
    ctx.potential_eval(pot, dev(P), out)
    assert rel(host(out).ravel(), g["pot_points"]) < 1e-12


@pytest.mark.parametrize("name", SCENARIOS)
def test_poisson(ctx, name):
    g, meta, _ = load_golden(name)
    nr, npl = meta["nr"], meta["np"]
    ar = dev(g["ar"])
    outs = [torch.zeros((nr, npl), dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.computePhil(ar, dev(g["guess_rhl"].reshape(nr, npl)), *outs)
    for o, key in zip(outs, ("guess_phil", "guess_Pr", "guess_Pr2")):
        assert rel_rows(host(o), g[key].reshape(nr, npl)) < TOL, key


@pytest.mark.parametrize("name", SCENARIOS)
def test_actions(ctx, name):
    g, meta, pts = load_golden(name)
    ar, tabs, pot = guess_pot(ctx, g, meta)
    delta = ctx.delta(dev(g["Egrid"]), dev(g["Dgrid"]))
    A = np.array([[float(x) for x in a[1:]] for a in pts if a[0] == "A"])
    out = torch.zeros((len(A), 2), dtype=torch.float64, device="cuda")
    ctx.uvOrb_actions(pot, delta, dev(A), out)
    assert rel(host(out).ravel(), g["actions"]) < TOL


@pytest.mark.parametrize("name", SCENARIOS)
def test_point_moments(ctx, name):
    g, meta, pts = load_golden(name)
    ar, tabs, pot = guess_pot(ctx, g, meta)
    delta = ctx.delta(dev(g["Egrid"]), dev(g["Dgrid"]))
    M = np.array([[float(a[1]), float(a[2])] for a in pts if a[0] == "M"])
    out = torch.zeros((6, len(M)), dtype=torch.float64, device="cuda")
    st = ctx.moments_points(pot, delta, df_of(meta), F.Rule(), dev(M), out)
    got = host(out).T
    ref = g["moments"].reshape(-1, 6)
    assert st.failures == 0
    assert rel(got[:, [0, 2, 3, 4]], ref[:, [0, 2, 3, 4]]) < TOL
    assert np.max(np.abs(got[:, 1] - ref[:, 1])) < 1e-7 * np.max(np.abs(ref[:, 2]))


@pytest.mark.parametrize("name", SCENARIOS)
def test_compute_new_phi(ctx, name):
    """One computeNewPhi (pot/potLeg.cpp:76-82) from the guess potential."""
    g, meta, _ = load_golden(name)
    nr, ng, npl = meta["nr"], meta["ng"], meta["np"]
    ar, tabs, pot = guess_pot(ctx, g, meta)
    delta = ctx.delta(dev(g["Egrid"]), dev(g["Dgrid"]))
    grids = torch.zeros((6, nr, ng), dtype=torch.float64, device="cuda")
    coef = torch.zeros((6, nr, npl), dtype=torch.float64, device="cuda")
    outs = [torch.zeros((nr, npl), dtype=torch.float64, device="cuda") for _ in range(3)]
    st = ctx.computeNewPhi(pot, delta, df_of(meta), F.Rule(), ng, grids, coef, *outs)
    assert st.failures == 0 and st.nodes == nr * ng * 22 ** 3
    c = host(coef)
    for q, key in ((0, "rhl"), (2, "sigRl"), (3, "sigpl"), (4, "sigzl")):
        assert rel_rows(c[q], g["it0_" + key].reshape(nr, npl)) < TOL, key
    for o, key in zip(outs, ("it0_phil", "it0_Pr", "it0_Pr2")):
        assert rel_rows(host(o), g[key].reshape(nr, npl)) < TOL, key
    # virial sums on the new potential vs the oracle restatement of vir2
    newpot = ctx.potential(ar, *outs)
    v = ctx.vir2(newpot, ng, coef)
    m1 = oracle_model(g, meta, host(outs[0]), host(outs[1]), host(outs[2]))
    vo = m1.vir2(c.reshape(6, -1))
    for key in ("KRR", "Kzz", "WRR", "Wzz", "pot"):
        if np.isnan(vo[key]):
            assert np.isnan(v[key])
        else:
            assert abs(v[key] - vo[key]) <= 1e-6 * abs(vo[key]), key


def test_run_model_two_iterations(ctx):
    """The whole one-component loop (fJmodels.cpp:86-144) vs the reference's second iteration."""
    g, meta, _ = load_golden("hern_dpl")
    nr, ng, npl = meta["nr"], meta["ng"], meta["np"]
    p = meta["p"]
    df = df_of(meta)
    # The focal-distance fit of the reference (delta/Delta.cpp) is not reproducible across
    # floating-point contraction settings, so the loop is run on the reference's own table.
    out = ctx.run_model(nr, ng, npl, meta["rmin"], meta["rmax"], df, F.Rule(), itermax=2,
                        delta_table=(g["Egrid"], g["Dgrid"]))
    assert out["iterations"] == 2 and out["failures"] == 0
    # After two iterations the first iteration's rounding-level differences (libm vs CUDA
    # exp/log/pow) have passed through the Poisson solve and a second moment sweep.  The
    # reference's own builds with and without FMA contraction, run on this fixture's
    # focal-distance table, differ by 1.9e-8 (first iteration) and 3e-9 (second) on its
    # outer shells (density below 1e-6 of the centre), where a few nodes decide the shell:
    # 2e-9 on the shells above that density, 1e-7 on the outer ones (single iterations keep
    # 1e-9 everywhere).
    ref = g["it1_rhl"].reshape(nr, npl)
    inner = np.abs(ref[:, 0]) >= 1e-6 * abs(ref[0, 0])
    assert rel_shells(out["coef6"][0][inner], ref[inner]) < 2 * TOL
    assert rel_shells(out["coef6"][0], ref) < 100 * TOL
    assert rel_shells(out["phil"], g["it1_phil"].reshape(nr, npl)) < 2 * TOL
    ref_vir = g["vir2"][1]  # KE, PE, W/K printed with %f after the second iteration
    K = out["vir7"][0] + out["vir7"][1]
    assert abs(out["vir7"][4] / K - ref_vir[4]) < 1.5e-6
    assert p["itermax"] == 2


@pytest.mark.parametrize("jquad", [8, 16])
def test_gauss_legendre_momentum_rule(ctx, jquad):
    """Fixed Gauss-Legendre momentum integrals: GPU vs the oracle with the same rule."""
    g, meta, pts = load_golden("hern_dpl")
    nr, npl = meta["nr"], meta["np"]
    ar, tabs, pot = guess_pot(ctx, g, meta)
    delta = ctx.delta(dev(g["Egrid"]), dev(g["Dgrid"]))
    A = np.array([[float(x) for x in a[1:]] for a in pts if a[0] == "A"])
    out = torch.zeros((len(A), 2), dtype=torch.float64, device="cuda")
    ctx.uvOrb_actions(pot, delta, dev(A), out, jquad=jquad)
    m = oracle_model(g, meta, g["guess_phil"].reshape(nr, npl), g["guess_Pr"].reshape(nr, npl),
                     g["guess_Pr2"].reshape(nr, npl), jquad=jquad)
    ref = []
    for R, z, vR, vp, vz in A:
        if 0.5 * (vR * vR + vp * vp + vz * vz) + m.phi(R, z) >= 0:
            ref += [-1, -1]
        else:
            ref += list(m.actions(R, z, vR, vp, vz))
    assert rel(host(out).ravel(), ref) < TOL


def test_tanh_sinh_rule_points(ctx):
    """The optional 22-point tanh-sinh velocity rule: GPU vs oracle with the same rule."""
    g, meta, _ = load_golden("hern_dpl")
    nr, npl = meta["nr"], meta["np"]
    ar, tabs, pot = guess_pot(ctx, g, meta)
    delta = ctx.delta(dev(g["Egrid"]), dev(g["Dgrid"]))
    x, w = F.tanh_sinh_rule(22)
    M = np.array([[0.8, 0.3], [3.0, 0.5]])
    out = torch.zeros((6, len(M)), dtype=torch.float64, device="cuda")
    ctx.moments_points(pot, delta, df_of(meta), F.Rule(x, w), dev(M), out)
    m = oracle_model(g, meta, g["guess_phil"].reshape(nr, npl), g["guess_Pr"].reshape(nr, npl),
                     g["guess_Pr2"].reshape(nr, npl), xq=x, wq=w)
    ref = np.array([m.rhofDF(R, z)[0] for R, z in M])
    got = host(out).T
    assert rel(got[:, [0, 2, 3, 4]], ref[:, [0, 2, 3, 4]]) < TOL


def test_c1_grid_subset(ctx):
    """Reference defaults of the first configuration (40 radii in 0.01..100, 20 polar
    nodes, l <= 8): GPU moments on a spread of grid points vs the oracle."""
    nr, ng, npl = 40, 20, 5
    ar = F.log_grid(0.01, 100.0, nr)
    rhl = F.guess_rhl(ar, ng, npl, "Hernquist")
    phil, Pr, Pr2 = O.compute_phil(ar, rhl)
    E, D, _ = F.tabulate_delta(ar, phil, Pr, Pr2)
    ci, _ = F.gauleg(0, 1, ng)
    idx = [(0, 0), (7, 3), (15, 10), (22, 19), (30, 5), (39, 12)]
    M = np.array([[ar[n] * np.sqrt(1 - ci[k] ** 2), ar[n] * ci[k]] for n, k in idx])
    pot = ctx.potential(dev(ar), dev(phil), dev(Pr), dev(Pr2))
    delta = ctx.delta(dev(E), dev(D))
    df = F.DFParams("Hernquist")
    out = torch.zeros((6, len(M)), dtype=torch.float64, device="cuda")
    st = ctx.moments_points(pot, delta, df, F.Rule(), dev(M), out)
    m = O.Model(ar, phil, Pr, Pr2, E, D, ng, alpha=1.667, beta=5.0)
    ref = np.array([m.rhofDF(R, z)[0] for R, z in M])
    got = host(out).T
    assert st.failures == 0
    assert rel(got[:, [0, 2, 3, 4]], ref[:, [0, 2, 3, 4]]) < TOL
