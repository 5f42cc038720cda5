"""The cumulative Poisson solve (FJ_POISSON_CUMULATIVE): the radial integrals of
computeInts (pot/Potential.cpp:82-155) taken exactly over the linear interpolation of
the density multipoles, as prefix sums.  Checked against the oracle's restatement,
which integrates each grid interval with a 24-point Gauss-Legendre rule instead of the
kernel's closed forms, and in a self-consistent loop, which converges below the
reference's stopping level with it (max |d phil / phil_0| < 1e-5)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402
from fjmodels_gb300 import _abi as A  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = F.Context(0)
    c.set_poisson(A.FJ_POISSON_CUMULATIVE)
    yield c
    c.close()


def _dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def _cases():
    rng = np.random.default_rng(11)
    for model, nr, npl, rmax in (("Hernquist", 40, 5, 100.0), ("NFW", 80, 7, 300.0), ("Isochrone", 96, 24, 100.0),
                                 ("NFW", 2, 1, 10.0)):
        ar = O.log_grid(1e-3, rmax, nr)
        rhl = O.guess_rhl(ar, 16, npl, model)
        if npl > 1:  # a flattened density: seeded multipoles l > 0
            rhl[1:, 1:] = rhl[1:, :1] * rng.uniform(-0.05, 0.05, size=(nr - 1, npl - 1))
        yield f"{model}-{nr}x{npl}", ar, rhl


@pytest.mark.parametrize("case", list(_cases()), ids=lambda c: c[0])
def test_cumulative_poisson_matches_oracle(cctx, case):
    _, ar, rhl = case
    nr, npl = rhl.shape
    outs = [torch.zeros((nr, npl), dtype=torch.float64, device="cuda") for _ in range(3)]
    cctx.computePhil(_dev(ar), _dev(rhl), *outs)
    ref = O.compute_phil(ar, rhl, cumulative=True)
    for o, r, name in zip(outs, ref, ("phil", "Pr", "Pr2")):
        got = o.cpu().numpy()
        scale = np.abs(r).max(axis=1, keepdims=True) + 1e-300
        err = float(np.max(np.abs(got - r) / scale))
        assert err < 1e-12, (name, err)


def test_loop_converges_with_cumulative_poisson(cctx):
    """A reduced rotating NFW model (32 x 12 grid, l <= 8, 16^3 nodes, mixed form) runs
    until max |d phil / phil_0| < 1e-5 well before its iteration limit."""
    x, w = F.tanh_sinh_rule(16)
    rule = F.Rule(x, w, precision=A.FJ_PREC_MIXED)
    df = F.DFParams("NFW", 0.55, 0.55, 1.0, 1.0, chi=1.0, k=0.5)
    r = cctx.run_model(32, 12, 5, 1e-3, 300.0, df, rule, itermax=60, tol=1e-5)
    assert r["iterations"] < 60 and r["last_change"] < 1e-5, r
    assert r["failures"] == 0
