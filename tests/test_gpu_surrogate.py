"""The action surrogate's tensor-core MLP: forward outputs and mean-squared-error
gradients against a float32 reference of the same network on the CPU (torch),
which rounds weights, activations and back-propagated errors to BF16 at the same
points as the GPU path; then training reduces the loss on a smooth target.

Tolerances: outputs 2e-3 of their scale; each layer's weight and bias gradients
1e-2 of the layer's largest gradient (BF16 rounding flips near ties and FP32
summation order)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402

pytestmark = pytest.mark.gpu
B = 1024


def gelu(z):
    return 0.5 * z * (1 + torch.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    u = 0.7978845608028654 * (z + 0.044715 * z ** 3)
    t = torch.tanh(u)
    return 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * 0.7978845608028654 * (1 + 3 * 0.044715 * z * z)


def bf(x):
    return x.bfloat16().float()


def reference(layers, X, T):
    """Forward, loss and gradients in float32 with the GPU's BF16 rounding points."""
    Wb = [bf(torch.tensor(W, dtype=torch.float32)) for W, _ in layers]
    bs = [torch.tensor(b, dtype=torch.float32) for _, b in layers]
    h = bf(X)
    Hs, Zs = [h], []
    for l in range(4):
        z = h @ Wb[l].T + bs[l]
        Zs.append(z)
        h = bf(gelu(z))
        Hs.append(h)
    y = h @ Wb[4].T + bs[4]
    d = y[:, :2] - T
    loss = (d * d).mean()
    dY = torch.zeros_like(y)
    dY[:, :2] = 2 * d / d.numel()
    dY = bf(dY)
    grads = [None] * 5
    grads[4] = (dY.T @ Hs[4], dY.sum(0))
    dz = bf((dY @ Wb[4]) * gelu_grad(Zs[3]))
    for l in range(3, -1, -1):
        grads[l] = (dz.T @ Hs[l], dz.sum(0))
        if l > 0:
            dz = bf((dz @ Wb[l]) * gelu_grad(Zs[l - 1]))
    return y, loss.item(), grads


def features(n, seed):
    g = torch.Generator().manual_seed(seed)
    X = torch.zeros(n, 16)
    X[:, :13] = torch.randn(n, 13, generator=g)
    T = torch.stack([torch.sin(X[:, 0]) + 0.5 * X[:, 1] ** 2, torch.cos(X[:, 2]) * X[:, 3]], 1)
    return X, T


def test_forward_and_gradients_vs_cpu(ctx):
    s = F.Surrogate(ctx, batch=B, seed=7)
    X, T = features(B, 3)
    Xd, Td = X.cuda(), T.contiguous().cuda()
    layers = s.unpack(s.params())
    y_ref, loss_ref, g_ref = reference(layers, X, T)
    Y = torch.zeros(B, 16, device="cuda")
    s.predict(Xd, Y)
    torch.cuda.synchronize()
    yc = Y.cpu()
    assert (yc[:, :2] - y_ref[:, :2]).abs().max().item() <= 2e-3 * y_ref[:, :2].abs().max().item() + 1e-6
    g, loss = s.gradients(Xd, Td)
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    for l, ((gW, gb), (W, b)) in enumerate(zip(s.unpack(g), layers)):
        rW, rb = g_ref[l]
        scale = max(rW.abs().max().item(), rb.abs().max().item())
        assert np.abs(gW - rW.numpy()).max() <= 1e-2 * scale, ("W", l)
        assert np.abs(gb - rb.numpy()).max() <= 1e-2 * scale, ("b", l)
    s.close()


def test_training_reduces_loss(ctx):
    s = F.Surrogate(ctx, batch=B, seed=11)
    X, T = features(64 * B, 5)
    Xd, Td = X.cuda(), T.contiguous().cuda()
    _, loss0 = s.gradients(Xd, Td)
    loss = s.train(Xd, Td, epochs=3, lr=2e-3)
    assert loss < 0.1 * loss0, (loss0, loss)
    # the frozen padding outputs stay exactly zero
    p = s.unpack(s.params())
    assert np.all(p[4][0][2:] == 0) and np.all(p[4][1][2:] == 0)
    s.close()


def _nfw_80_tanh():
    nr, ng, npl = 80, 40, 7
    ar = F.log_grid(1e-3, 300.0, nr)
    from oracle import oracle as O
    phil, Pr, Pr2 = O.compute_phil(ar, F.guess_rhl(ar, ng, npl, "NFW"))
    E, D, _ = F.tabulate_delta(ar, phil, Pr, Pr2)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")  # noqa: E731
    return (nr, ng, npl), [dev(t) for t in (ar, phil, Pr, Pr2)], (dev(E), dev(D))


def test_surrogate_moments_gain(ctx):
    """Fit to one exact iteration of the 80 x 40 rotating NFW workload (22^3 tanh-sinh
    nodes), then the surrogate's grid of moments.  What the trained network gains over the
    same network untrained: its densities' median error falls from 100 % to 8 %; over the
    exact kernel: the fused tensor-core kernel (equal to the separate passes) is > 20x
    faster.  The accuracy (median 8 %, 90th percentile 63 % measured) is what keeps it out
    of the chosen form: as a warm start it saves no exact iterations."""
    from fjmodels_gb300 import _abi as A
    (nr, ng, npl), tabs, (E, D) = _nfw_80_tanh()
    pot, delta = ctx.potential(*tabs), ctx.delta(E, D)
    df = F.DFParams("NFW", chi=1.0, k=0.5)
    rule = F.Rule(*F.tanh_sinh_rule(22), precision=A.FJ_PREC_MIXED)
    npts, nq3 = nr * ng, 22 ** 3
    jout = torch.empty(npts * nq3 * 2, dtype=torch.float32, device="cuda")
    g_exact = torch.zeros((6, nr, ng), dtype=torch.float64, device="cuda")
    ctx.set_action_output(jout)
    st = ctx.moments(pot, delta, df, rule, ng, g_exact)
    ctx.set_action_output(None)
    b = g_exact[0].cpu().numpy().ravel()
    untrained = F.Surrogate(ctx, batch=8192, seed=3)
    g_un = torch.zeros_like(g_exact)
    untrained.moments(pot, df, rule, ng, g_un)
    torch.cuda.synchronize()
    rel_un = np.abs(g_un[0].cpu().numpy().ravel() - b) / b
    untrained.close()
    s = F.Surrogate(ctx, batch=8192, seed=3)
    loss = s.fit(pot, df, ng, rule, jout, 1 << 20, seed=5, epochs=24, lr=2e-3, rho=g_exact[0].reshape(-1))
    g_sg = torch.zeros_like(g_exact)
    g_unf = torch.zeros_like(g_exact)
    s.moments(pot, df, rule, ng, g_sg)  # warm-up (workspace allocation)
    ms = s.moments(pot, df, rule, ng, g_sg)
    ms_unf = s.moments(pot, df, rule, ng, g_unf, fused=False)
    torch.cuda.synchronize()
    # the fused kernel and the separate passes (features, GEMMs, sums) agree
    ru = g_unf[0].cpu().numpy().ravel()
    print(f"fused {ms:.2f} ms, unfused {ms_unf:.1f} ms, max rel diff "
          f"{np.max(np.abs(g_sg[0].cpu().numpy().ravel() - ru) / ru):.2e}")
    assert np.max(np.abs(g_sg[0].cpu().numpy().ravel() - ru) / ru) < 1e-3
    assert ms < st.kernel_ms / 20
    rel = np.abs(g_sg[0].cpu().numpy().ravel() - b) / b
    print(f"surrogate: fit loss {loss:.3e}, moments {ms:.1f} ms vs exact {st.kernel_ms:.1f} ms, rho rel err median "
          f"{np.median(rel):.2e} p90 {np.percentile(rel, 90):.2e} (untrained: median {np.median(rel_un):.2e})")
    assert np.median(rel) < 0.12 and np.percentile(rel, 90) < 0.8
    assert np.median(rel) < 0.5 * np.median(rel_un)
    s.close()


def test_surrogate_schedule(ctx):
    """The surrogate as a warm start of the loop, on a smaller NFW model: an exact first
    iteration (the fit), three surrogate iterations (no audit fallback), then exact
    iterations until converged.  The converged model is the exact loop's (density
    multipoles within 1e-4); the exact iterations it takes are printed next to the exact
    loop's: the surrogate saves none on this workload (it is not part of the chosen form)."""
    from fjmodels_gb300 import _abi as A
    from tests.helpers import rel_rows
    rule = F.Rule(*F.tanh_sinh_rule(16), precision=A.FJ_PREC_MIXED)
    df = F.DFParams("NFW", chi=1.0, k=0.5)
    args = (40, 16, 5, 1e-3, 300.0, df, rule)
    ctx.set_poisson(A.FJ_POISSON_CUMULATIVE)
    try:
        ref = ctx.run_model(*args, itermax=100, tol=1e-5)
        s = F.Surrogate(ctx, batch=4096, seed=9)
        S, T = 3, 60
        out, rep = ctx.run_model_surrogate(*args, itermax=1 + S + T, surrogate=s, tol=1e-5, samples=1 << 18,
                                           epochs_first=8, epochs=8, lr=2e-3, exact_first=1, exact_last=T,
                                           audit_stride=50, audit_tol=10.0)
        s.close()
    finally:
        ctx.set_poisson(A.FJ_POISSON_QAGS)
    print(f"exact loop: {ref['iterations']} iterations; warm start: {rep['surrogate_iterations']} surrogate + "
          f"{out['iterations'] - rep['surrogate_iterations']} exact; report {rep}")
    assert rep["surrogate_iterations"] == S and rep["fallback_iterations"] == 0 and rep["fits"] == 1
    assert out["last_change"] < 1e-5 and out["iterations"] < 1 + S + T
    assert rel_rows(out["coef6"][0], ref["coef6"][0]) < 1e-4
