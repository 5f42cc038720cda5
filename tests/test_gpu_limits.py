"""The size limits of the C ABI: the largest sizes it takes give the oracle's results,
and arguments outside them are refused with FJ_ERR_ARG before any GPU work (FJError
in the Python mirror).

- npoly = 24 (l <= 46, the largest multipole order of fj_potential): the Poisson solve
  and the phase-space moments of a flattened model (axis ratio 0.7, so every even
  multipole is present) against the oracle, 1e-9 as in the parity tests; the mixed
  form against the plain FP64 form within the 1e-4 density bound of the chosen form.
- nq = 64 (the largest velocity rule): the moments of one point against the oracle.
- Refused: nr < 11, npoly > 24, nq > 64, no points, ngauss < 1, the mixed form with
  the quasi-isothermal DF.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402
from fjmodels_gb300 import _abi as A  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.helpers import rel, rel_rows  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = 1e-9


def dev(a):
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = F.Context(0)
    yield c
    c.close()


def _flattened(nr, npl, ng=32):
    ar = F.log_grid(0.01, 100.0, nr)
    rhl = F.guess_rhl(ar, ng, npl, "Hernquist", q=0.7)
    phil, Pr, Pr2 = O.compute_phil(ar, rhl)
    E, D, _ = F.tabulate_delta(ar, phil, Pr, Pr2)
    return ar, rhl, (phil, Pr, Pr2), (E, D)


def test_largest_multipole_order(ctx):
    nr, npl = 40, 24
    ar, rhl, tabs, (E, D) = _flattened(nr, npl)
    assert np.all(np.abs(rhl[nr // 2, 1:]) > 0)  # every even multipole is present
    outs = [torch.zeros((nr, npl), dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.computePhil(dev(ar), dev(rhl), *outs)
    for o, r, name in zip(outs, tabs, ("phil", "Pr", "Pr2")):
        assert rel_rows(host(o), r) < TOL, name
    pot = ctx.potential(dev(ar), *[dev(t) for t in tabs])
    delta = ctx.delta(dev(E), dev(D))
    df = F.DFParams("Hernquist")
    x, w = F.tanh_sinh_rule(22)
    M = np.array([[0.3, 0.2], [2.0, 1.5]])
    m = O.Model(ar, *tabs, E, D, 32, alpha=1.667, beta=5.0, xq=x, wq=w)
    ref = np.array([m.rhofDF(R, z)[0] for R, z in M])
    plain = torch.zeros((6, len(M)), dtype=torch.float64, device="cuda")
    st = ctx.moments_points(pot, delta, df, F.Rule(x, w), dev(M), plain)
    got = host(plain).T
    assert st.failures == 0
    assert rel(got[:, [0, 2, 3, 4]], ref[:, [0, 2, 3, 4]]) < TOL
    mixed = torch.zeros((6, len(M)), dtype=torch.float64, device="cuda")
    ctx.moments_points(pot, delta, df, F.Rule(x, w, precision=A.FJ_PREC_MIXED), dev(M), mixed)
    assert rel(host(mixed).T[:, 0], got[:, 0]) < 1e-4


def test_largest_velocity_rule(ctx):
    nr, npl = 24, 3
    ar, rhl, tabs, (E, D) = _flattened(nr, npl, ng=8)
    pot = ctx.potential(dev(ar), *[dev(t) for t in tabs])
    delta = ctx.delta(dev(E), dev(D))
    x, w = F.gauleg(-1.0, 1.0, 64)
    M = np.array([[1.0, 0.5]])
    out = torch.zeros((6, 1), dtype=torch.float64, device="cuda")
    st = ctx.moments_points(pot, delta, F.DFParams("Hernquist"), F.Rule(x, w), dev(M), out)
    assert st.nodes == 64 ** 3
    m = O.Model(ar, *tabs, E, D, 8, alpha=1.667, beta=5.0, xq=x, wq=w)
    ref = m.rhofDF(1.0, 0.5)[0]
    got = host(out)[:, 0]
    assert rel(got[[0, 2, 3, 4]], ref[[0, 2, 3, 4]]) < TOL


def test_arguments_outside_the_limits(ctx):
    ar, rhl, tabs, (E, D) = _flattened(24, 3, ng=8)
    delta = ctx.delta(dev(E), dev(D))
    df = F.DFParams("Hernquist")
    pts = dev(np.array([[1.0, 0.5]]))
    out = torch.zeros((6, 1), dtype=torch.float64, device="cuda")
    ok = ctx.potential(dev(ar), *[dev(t) for t in tabs])
    short = ctx.potential(dev(ar[:10]), *[dev(t[:10]) for t in tabs])
    wide = np.zeros((24, 25))
    too_many = ctx.potential(dev(ar), dev(wide), dev(wide), dev(wide))
    x65, w65 = F.gauleg(-1.0, 1.0, 65)
    qiso = F.DFParams("Hernquist", kind=1)
    cases = [
        (short, df, F.Rule(), pts),
        (too_many, df, F.Rule(), pts),
        (ok, df, F.Rule(x65, w65), pts),
        (ok, df, F.Rule(), dev(np.zeros((0, 2)))),
        (ok, qiso, F.Rule(precision=A.FJ_PREC_MIXED), pts),
    ]
    for i, (pot, d, rule, p) in enumerate(cases):
        with pytest.raises(F.FJError):
            ctx.moments_points(pot, delta, d, rule, p, out)
            pytest.fail(f"case {i} accepted")
    grids = torch.zeros((6, 24, 1), dtype=torch.float64, device="cuda")
    with pytest.raises(F.FJError):
        ctx.moments(ok, delta, df, F.Rule(), 0, grids)
    assert np.all(host(out) == 0)  # nothing was launched
    ctx.moments_points(ok, delta, df, F.Rule(), pts, out)  # the context still works
    assert host(out)[0, 0] > 0
