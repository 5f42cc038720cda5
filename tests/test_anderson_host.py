"""Anderson mixing on host tables (fj_anderson_create / fj_anderson_host_step, the same
update fj_anderson_step applies to device tables), on the CPU: a linear contraction,
the divergence restart, the arguments, and the self-consistent loop of the reference's
FP64 algorithm (the oracle, the cumulative Poisson solve) iterated plain and mixed.
The reference iterates the plain map (fJmodels.cpp:131-143)."""
import numpy as np
import pytest

import fjmodels_gb300 as F
from oracle import oracle as O


def _tables(nr=16, npl=3, seed=1):
    g = np.random.default_rng(seed)
    xs = g.uniform(-1.0, 1.0, (3, nr, npl))
    xs[0, :, 0] = -1.0 - g.uniform(0, 1, nr)  # the potential's monopole: the stopping test's scale
    return xs


@pytest.mark.parametrize("beta", [1.0, 1.6])
def test_linear_map(beta):
    """A contraction with rates 0.6 (monopoles) and 0.3: depth 2 reaches the fixed point to
    rounding within 10 steps; the first step has no history: x + beta (g - x)."""
    nr, npl = 16, 3
    xs = _tables(nr, npl)
    rate = np.full((3, nr, npl), 0.6)
    rate[:, :, 1:] = 0.3
    x = np.zeros_like(xs)
    x[0, :, 0] = -1.0
    a = F.Anderson(2, beta)
    g = xs + rate * (x - xs)
    x0 = x.copy()
    a.step(x, g)
    assert np.allclose(x, x0 + beta * (g - x0), rtol=0, atol=1e-15)
    for _ in range(9):
        g = xs + rate * (x - xs)
        ch = a.step(x, g)
    assert ch < 1e-12 and np.max(np.abs(x - xs)) < 1e-12
    a.close()


def test_restart_when_diverging():
    """A change more than twice the last drops the history: that step is x + beta (g - x)."""
    xs = _tables(12, 2, seed=3)
    x = xs.copy()
    x[0] += 1e-3
    a = F.Anderson(2)
    for _ in range(3):
        a.step(x, xs + 0.5 * (x - xs))
    g = x + 1.0
    g[0, :, 0] = x[0, :, 0] - 0.5
    assert a.step(x, g) > 0.1 and np.array_equal(x, g)


def test_arguments():
    for depth, beta in ((9, 1.0), (-1, 1.0), (2, 0.0), (2, 4.5)):
        with pytest.raises(F.FJError):
            F.Anderson(depth, beta)
    a = F.Anderson(2)
    with pytest.raises(F.FJError):
        a.step(np.zeros((3, 4, 2)), np.zeros((3, 4, 3)))
    with pytest.raises(F.FJError):
        a.step(np.zeros((3, 4, 2), dtype=np.float32), np.zeros((3, 4, 2)))


def _oracle_model():
    """A 16 x 3 Hernquist model (l <= 4), the 12-point tanh-sinh velocity rule, the Delta table
    of the guess potential; G maps potential tables [3][nr][npoly] to the next ones."""
    nr, ng, npl = 16, 3, 3
    ar = F.log_grid(0.01, 100.0, nr)
    x0 = np.array(O.compute_phil(ar, F.guess_rhl(ar, ng, npl, "Hernquist"), cumulative=True))
    E, D, _ = F.tabulate_delta(ar, *x0)
    xq, wq = F.tanh_sinh_rule(12)

    def G(x):
        m = O.Model(ar, x[0], x[1], x[2], E, D, ng, alpha=1.667, beta=5.0, xq=xq, wq=wq)
        c, _ = O.project6(ar, ng, npl, m.moment_grid()[0])
        return np.array(O.compute_phil(ar, c[0].reshape(nr, npl), cumulative=True))

    return x0, G


def _change(x, g):
    return float(np.max(np.abs(g[0] - x[0]) / np.abs(g[0][:, :1])))


def test_oracle_loop_mixed_reaches_the_plain_fixed_point():
    """The reference's algorithm (oracle, FP64): the plain loop to a change of 1e-7 (about 40
    iterations) and the depth-2 mixed loop (factors 1 and 1.6) to a change of 1e-6 followed by
    a confirming plain step: the mixed loops stop in fewer than half the iterations the plain
    loop needs to 1e-6, at the plain loop's fixed point (within 1e-5 of the monopole)."""
    x0, G = _oracle_model()
    x, plain_to_1e6 = x0.copy(), None
    for k in range(80):
        g = G(x)
        ch = _change(x, g)
        if plain_to_1e6 is None and ch < 1e-6:
            plain_to_1e6 = k + 1
        x = g
        if ch < 1e-7:
            break
    fixed = x
    assert plain_to_1e6 is not None
    for beta in (1.0, 1.6):
        a, x, confirmed = F.Anderson(2, beta), x0.copy(), False
        for k in range(40):
            g = G(x)
            ch = _change(x, g)
            if ch < 1e-6:
                if confirmed:
                    break
                confirmed, x = True, g
                continue
            confirmed = False
            a.step(x, g)
        its = k + 1
        d = float(np.max(np.abs(g[0] - fixed[0]) / np.abs(fixed[0][:, :1])))
        print(f"beta {beta}: {its} iterations (plain: {plain_to_1e6} to 1e-6), potential vs the plain fixed point {d:.1e}")
        assert ch < 1e-6 and its < plain_to_1e6 / 2 and d < 1e-5
