"""Projected density, line-of-sight profiles and velocity distributions on the GPU
(fj_los: SigmaDF, line_profile, P_vp, P_vz, P_vr of integ/Integ.cpp:168-220) against
the reference's own values in the golden fixtures and against the oracle on the
rotating NFW 80 x 40 model.  Tolerances: 1e-10 relative to the fixtures (the reference
sums its tensor rules in OpenMP order; the GPU path is the FP64 phase-space path that
matches the oracle's moments to ~1e-12), 1e-9 against the oracle on the larger model
(adaptive quadrature decisions at rounding-level ties).  Also the reference's
line-profile file layout and argument errors."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402
from fjmodels_gb300 import _abi as A  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.conftest import load_golden  # noqa: E402
from tests.helpers import oracle_model, rel  # noqa: E402
from tests.test_oracle_golden import los_items  # noqa: E402

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def _df(meta):
    p = meta["p"]
    kind = A.FJ_DF_QUASIISO if meta["df"] == "qiso" else A.FJ_DF_DPL
    return F.DFParams(p["model"], p["dphi_h"], p["dz_h"], p["dphi_g"], p["dz_g"], p["chi"], p["mass"], p["r0"],
                      k=meta["k"], kind=kind)


def _gpu_los(ctx, pot, delta, df, rule, rhl, items):
    out = np.zeros(len(items))
    for kind in sorted({it[0] for it in items}):
        idx = [i for i, it in enumerate(items) if it[0] == kind]
        rzv = dev([[items[i][1], items[i][2], items[i][3]] for i in idx])
        o = torch.zeros(len(idx), dtype=torch.float64, device="cuda")
        ctx.los(pot, delta, df, rule, rhl, kind, rzv, o)
        out[idx] = o.cpu().numpy()
    return out


@pytest.mark.parametrize("name", ["hern_dpl", "nfw_dpl_rot", "hern_qiso"])
def test_los_matches_reference(ctx, name):
    g, meta, pts = load_golden(name)
    nr, npl = meta["nr"], meta["np"]
    pot = ctx.potential(dev(g["ar"]), dev(g["guess_phil"]), dev(g["guess_Pr"]), dev(g["guess_Pr2"]))
    delta = ctx.delta(dev(g["Egrid"]), dev(g["Dgrid"]))
    items = los_items(pts)
    got = _gpu_los(ctx, pot, delta, _df(meta), F.Rule(), dev(g["guess_rhl"].reshape(nr, npl)), items)
    assert rel(got, g["los"]) < 1e-10, np.abs(got / g["los"] - 1)


def test_los_matches_oracle_nfw_80():
    """Rotating NFW 80 x 40 (l <= 12) in its guess potential: every kind at a few points
    from the centre to the outer shells."""
    c = F.Context(0)
    nr, ng, npl = 80, 40, 7
    ar = F.log_grid(1e-3, 300.0, nr)
    rhl = F.guess_rhl(ar, ng, npl, "NFW")
    phil, Pr, Pr2 = O.compute_phil(ar, rhl)
    E, D, _ = F.tabulate_delta(ar, phil, Pr, Pr2)
    pot = c.potential(dev(ar), dev(phil), dev(Pr), dev(Pr2))
    delta = c.delta(dev(E), dev(D))
    df = F.DFParams("NFW", chi=1.0, k=0.5)
    m = O.Model(ar, phil, Pr, Pr2, E, D, ng, df_kind=O.DF_DPL, alpha=1.667, beta=3.0, mass=1.0, r0=1.0,
                dphi_h=0.55, dz_h=0.55, dphi_g=1.0, dz_g=1.0, chi=1.0, k=0.5)
    items = []
    for R, z in ((0.01, 0.005), (1.0, 0.5), (20.0, 3.0)):
        items.append((O.LOS_SIGMA, R, z, 0.0))
        items.append((O.LOS_LINE, R, z, 0.2))
        items.append((O.LOS_PVPHI, R, z, 0.1))
        items.append((O.LOS_PVZ, R, z, -0.05))
        items.append((O.LOS_PVR, R, z, 0.15))
    got = _gpu_los(c, pot, delta, df, F.Rule(), dev(rhl), items)
    ref = np.array([m.los(rhl, *it) for it in items])
    assert np.all(ref > 0) and rel(got, ref) < 1e-9, np.abs(got / ref - 1)
    c.close()


def test_line_profile_file_layout(ctx, tmp_path):
    """writeOut's line-profile block: 150 rows, three (v, profile) pairs, the profile of each
    pair the LINE value at that velocity."""
    g, meta, pts = load_golden("hern_dpl")
    nr, npl = meta["nr"], meta["np"]
    pot = ctx.potential(dev(g["ar"]), dev(g["guess_phil"]), dev(g["guess_Pr"]), dev(g["guess_Pr2"]))
    delta = ctx.delta(dev(g["Egrid"]), dev(g["Dgrid"]))
    rhl = dev(g["guess_rhl"].reshape(nr, npl))
    f = tmp_path / "m.lp"
    lp = ctx.line_profile_file(str(f), pot, delta, _df(meta), F.Rule(), rhl)
    rows = [list(map(float, line.split())) for line in f.read_text().splitlines()]
    assert len(rows) == 150 and all(len(r) == 6 for r in rows)
    assert lp.shape == (3, 150) and np.all(np.isfinite(lp))
    assert np.allclose([r[1] for r in rows], lp[0], rtol=1e-5)
    v = np.array([r[0] for r in rows])
    assert np.all(np.diff(v) > 0) and v[0] < 0 < v[-1]


def test_los_arguments(ctx):
    g, meta, _ = load_golden("hern_dpl")
    pot = ctx.potential(dev(g["ar"]), dev(g["guess_phil"]), dev(g["guess_Pr"]), dev(g["guess_Pr2"]))
    delta = ctx.delta(dev(g["Egrid"]), dev(g["Dgrid"]))
    rzv = dev([[1.0, 0.5, 0.1]])
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    with pytest.raises(F.FJError):
        ctx.los(pot, delta, _df(meta), F.Rule(), None, A.FJ_LOS_LINE, rzv, out)  # SigmaDF needs rhl
    with pytest.raises(F.FJError):
        ctx.los(pot, delta, _df(meta), F.Rule(), None, 9, rzv, out)
    with pytest.raises(F.FJError):
        ctx.los(pot, delta, _df(meta), F.Rule(precision=A.FJ_PREC_MIXED), None, A.FJ_LOS_PVZ, rzv, out)
