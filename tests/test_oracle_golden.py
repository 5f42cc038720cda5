"""The CPU oracle against fixtures produced by the reference's own sources
(tests/golden/make_golden.py): potential, Poisson, focal-distance table,
actions, moments, one full iteration's coefficients and the virial sums."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import load_golden
from tests.helpers import _nan_diff, oracle_model, rel, rel_rows

SCENARIOS = ["hern_dpl", "nfw_dpl_rot", "hern_qiso"]


@pytest.mark.parametrize("name", SCENARIOS)
def test_setup_matches_reference(name):
    g, meta, pts = load_golden(name)
    nr, ng, npl = meta["nr"], meta["ng"], meta["np"]
    p = meta["p"]
    ar = O.log_grid(meta["rmin"], meta["rmax"], nr)
    assert rel(ar, g["ar"]) == 0.0
    rhl = O.guess_rhl(ar, ng, npl, p["model"], p["mass"], p["r0"])
    assert rel_rows(rhl, g["guess_rhl"].reshape(nr, npl)) < 1e-14
    phil, Pr, Pr2 = O.compute_phil(ar, rhl)
    for a, key in ((phil, "guess_phil"), (Pr, "guess_Pr"), (Pr2, "guess_Pr2")):
        assert rel_rows(a, g[key].reshape(nr, npl)) < 1e-13, key
    m = oracle_model(g, meta, phil, Pr, Pr2)
    P = [(float(a[1]), float(a[2])) for a in pts if a[0] == "P"]
    pv = np.array([[m.phi(R, z), m.dR(R, z), m.dz(R, z)] for R, z in P]).ravel()
    assert rel(pv, g["pot_points"]) < 1e-13
    E, D, fail = m.tabulate_delta(30)
    assert rel(E, g["Egrid"]) < 1e-12 and rel(D, g["Dgrid"]) < 1e-9


@pytest.mark.parametrize("name", SCENARIOS)
def test_actions_match_reference(name):
    g, meta, pts = load_golden(name)
    nr, npl = meta["nr"], meta["np"]
    m = oracle_model(g, meta, g["guess_phil"].reshape(nr, npl), g["guess_Pr"].reshape(nr, npl),
                     g["guess_Pr2"].reshape(nr, npl))
    out = []
    for a in pts:
        if a[0] != "A":
            continue
        R, z, vR, vp, vz = map(float, a[1:])
        Phi = m.phi(R, z)
        if 0.5 * (vR * vR + vp * vp + vz * vz) + Phi >= 0:
            out += [-1, -1]
        else:
            out += list(m.actions(R, z, vR, vp, vz))
    assert rel(out, g["actions"]) < 1e-10


@pytest.mark.parametrize("name", SCENARIOS)
def test_point_moments_match_reference(name):
    g, meta, pts = load_golden(name)
    nr, npl = meta["nr"], meta["np"]
    m = oracle_model(g, meta, g["guess_phil"].reshape(nr, npl), g["guess_Pr"].reshape(nr, npl),
                     g["guess_Pr2"].reshape(nr, npl))
    M = [(float(a[1]), float(a[2])) for a in pts if a[0] == "M"]
    got = np.array([m.rhofDF(R, z)[0] for R, z in M])
    ref = g["moments"].reshape(-1, 6)
    # rho and the even second moments to rounding; vrot/sigRz are differences of
    # near-cancelling sums (the reference sums them in OpenMP order)
    assert rel(got[:, [0, 2, 3, 4]], ref[:, [0, 2, 3, 4]]) < 1e-12
    assert np.max(np.abs(got[:, 1] - ref[:, 1])) < 1e-8 * np.max(np.abs(ref[:, 2]))


@pytest.mark.parametrize("name", SCENARIOS)
def test_first_iteration_matches_reference(name):
    g, meta, pts = load_golden(name)
    nr, ng, npl = meta["nr"], meta["ng"], meta["np"]
    m = oracle_model(g, meta, g["guess_phil"].reshape(nr, npl), g["guess_Pr"].reshape(nr, npl),
                     g["guess_Pr2"].reshape(nr, npl))
    grids, st = m.moment_grid()
    assert st["failures"] == 0
    coef, _ = O.project6(g["ar"], ng, npl, grids)
    for q, key in enumerate(("rhl", "sigRl", "sigpl", "sigzl")):
        qq = {"rhl": 0, "sigRl": 2, "sigpl": 3, "sigzl": 4}[key]
        assert rel_rows(coef[qq], g["it0_" + key].reshape(nr, npl)) < 1e-12, key
    phil, Pr, Pr2 = O.compute_phil(g["ar"], coef[0].reshape(nr, npl))
    for a, key in ((phil, "it0_phil"), (Pr, "it0_Pr"), (Pr2, "it0_Pr2")):
        assert rel_rows(a, g[key].reshape(nr, npl)) < 1e-11, key
    # virial sums (printed by the reference with %f)
    m1 = oracle_model(g, meta, phil, Pr, Pr2)
    v = m1.vir2(coef)
    K = v["KRR"] + v["Kzz"]
    mine = [v["mass_pr"], v["mass_sum"], K, v["pot"], v["pot"] / K, v["KRR"], v["WRR"], v["WRR"] / v["KRR"],
            v["Kzz"], v["Wzz"], v["Wzz"] / v["Kzz"]]
    assert np.max(_nan_diff(np.array(mine), g["vir2"][0])) < 1.5e-6


LOS_KINDS = {"S": O.LOS_SIGMA, "L": O.LOS_LINE, "F": O.LOS_PVPHI, "Z": O.LOS_PVZ, "X": O.LOS_PVR}


def los_items(pts):
    """(kind, R, z, v) of the projected-density, line-profile and velocity-distribution
    points, in fixture order."""
    return [(LOS_KINDS[a[0]], float(a[1]), float(a[2]), float(a[3]) if len(a) > 3 else 0.0)
            for a in pts if a[0] in LOS_KINDS]


@pytest.mark.parametrize("name", SCENARIOS)
def test_line_profiles_and_velocity_distributions_match_reference(name):
    """SigmaDF, line_profile, P_vp, P_vz, P_vr (integ/Integ.cpp:168-220) in the guess
    potential with the guess density multipoles; the reference sums its tensor rules in
    OpenMP order, so agreement is to rounding (1e-12 relative)."""
    g, meta, pts = load_golden(name)
    nr, npl = meta["nr"], meta["np"]
    m = oracle_model(g, meta, g["guess_phil"].reshape(nr, npl), g["guess_Pr"].reshape(nr, npl),
                     g["guess_Pr2"].reshape(nr, npl))
    items = los_items(pts)
    got = np.array([m.los(g["guess_rhl"].reshape(nr, npl), *it) for it in items])
    ref = g["los"]
    assert len(items) == len(ref) == 11
    assert np.all(np.isfinite(ref)) and np.all(ref > 0)
    assert rel(got, ref) < 1e-12, np.abs(got / ref - 1)


def test_tanh_sinh_table_is_the_reference_table():
    """orc_tanh_sinh01 regenerates include/GaussPts.h's 22-point [0,1] table from the
    tanh-sinh formula (h = 2/11, 12 significant digits): symmetric about 1/2 and
    integrating polynomials on [0, 1]."""
    x, w = O.tanh_sinh01()
    assert np.all(np.diff(x) > 0) and x[11] == 0.5 and abs(w.sum() - 1) < 4e-5  # the table stops at k = 10 and -11
    assert np.allclose(x[1:] + x[:0:-1], 1, atol=2e-12)


def test_two_component_reference_order_matches_reference():
    """The reference's two-component loop (twoComp, fJmodels.cpp:38-81), first iteration:
    component 1's moments in the total guess potential; its own potential, which replaces
    the total (Potential.cpp:182-188); component 2's moments in that; the total potential
    the sum of the two (updatePhil, potLeg.cpp:21-29).  The oracle composes the same
    sequence from its one-component pieces."""
    g, meta, _ = load_golden("twocomp_ref")
    nr, ng, npl = meta["nr"], meta["ng"], meta["np"]
    p, p2 = meta["p"], meta["p2"]
    ar = g["ar"]
    r1 = O.guess_rhl(ar, ng, npl, p["model"], p["mass"], p["r0"])
    r2 = O.guess_rhl(ar, ng, npl, p2["model"], p2["mass"], p2["r0"])
    assert rel_rows(r1, g["c1_guess_rhl"].reshape(nr, npl)) < 1e-14
    assert rel_rows(r2, g["c2_guess_rhl"].reshape(nr, npl)) < 1e-14
    total = [a + b for a, b in zip(O.compute_phil(ar, r1), O.compute_phil(ar, r2))]
    for a, key in zip(total, ("guess_phil", "guess_Pr", "guess_Pr2")):
        assert rel_rows(a, g[key].reshape(nr, npl)) < 1e-13, key
    m1 = oracle_model(g, meta, *total)
    grids, st = m1.moment_grid()
    assert st["failures"] == 0
    c1, _ = O.project6(ar, ng, npl, grids)
    pot1 = O.compute_phil(ar, c1[0].reshape(nr, npl))
    meta2 = dict(meta, p=p2)
    for a, key in zip(pot1, ("phil", "Pr", "Pr2")):
        assert rel_rows(a, g["it0_c1_" + key].reshape(nr, npl)) < 1e-11, key
    for q, key in ((0, "rhl"), (2, "sigRl"), (3, "sigpl"), (4, "sigzl")):
        assert rel_rows(c1[q], g["it0_c1_" + key].reshape(nr, npl)) < 1e-12, key
    # component 2's step on its own: its moments in the reference's component-1 potential
    ref_pot1 = [g["it0_c1_" + k].reshape(nr, npl) for k in ("phil", "Pr", "Pr2")]
    grids2, st2 = oracle_model(g, meta2, *ref_pot1).moment_grid()
    assert st2["failures"] == 0
    c2, _ = O.project6(ar, ng, npl, grids2)
    for q, key in ((0, "rhl"), (2, "sigRl"), (3, "sigpl"), (4, "sigzl")):
        assert rel_rows(c2[q], g["it0_c2_" + key].reshape(nr, npl)) < 1e-12, key
    pot2 = O.compute_phil(ar, c2[0].reshape(nr, npl))
    for a, b, key in zip(ref_pot1, pot2, ("phil", "Pr", "Pr2")):
        assert rel_rows(a + b, g["it0_" + key].reshape(nr, npl)) < 1e-11, key
    # the whole chain from the oracle's own component-1 potential, which differs from the
    # reference's at 1e-12 (moment sums in OpenMP order): the halo's adaptive quadrature
    # passes that on at up to ~1e-10
    grids2c, _ = oracle_model(g, meta2, *pot1).moment_grid()
    c2c, _ = O.project6(ar, ng, npl, grids2c)
    for q, key in ((0, "rhl"), (2, "sigRl"), (3, "sigpl"), (4, "sigzl")):
        assert rel_rows(c2c[q], g["it0_c2_" + key].reshape(nr, npl)) < 5e-10, key
