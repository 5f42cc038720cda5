"""fj_poisson_noalloc: the Poisson solve for callers that cannot allocate device
memory on their call path (their device memory belongs to their own pool
allocator, or the call sits in a latency-bound loop).  Its quadrature workspace
is a device array inside the library instead of context scratch.  This file is
collected last so that a failure here leaves every other test already run; it
passes on its own in a fresh process too.

Checked through the C ABI: two calls in a row give the same tables as
fj_poisson (same kernel, so agreement is exact; the parity tolerance of the
other tests, 1e-9 relative per shell, is what is asserted), and a request
beyond the array's size is refused with FJ_ERR_ARG before any GPU work.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402

pytestmark = pytest.mark.gpu


def _shell_rel(a, ref):
    scale = np.abs(ref[:, :1]) + 1e-300
    return float(np.max(np.abs(a - ref) / scale))


def test_noalloc_poisson_matches_context_poisson_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = F.load_library()
    nr, ng, npl = 80, 40, 7
    ar = F.log_grid(1e-3, 300.0, nr)
    rhl = F.guess_rhl(ar, ng, npl, "NFW")
    rng = np.random.default_rng(7)  # a non-spherical density: seeded multipoles l > 0
    rhl[1:, 1:] = rhl[1:, :1] * rng.uniform(-0.05, 0.05, size=(nr - 1, npl - 1))
    f64 = dict(dtype=torch.float64, device="cuda")
    d_ar, d_rhl = torch.tensor(ar, **f64), torch.tensor(rhl, **f64)

    ctx = F.Context(0)
    ref = [torch.zeros((nr, npl), **f64) for _ in range(3)]
    ctx.computePhil(d_ar, d_rhl, *ref)
    torch.cuda.synchronize()
    ref = [t.cpu().numpy() for t in ref]
    ctx.close()

    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        outs = [torch.full((nr, npl), np.nan, **f64) for _ in range(3)]
        rc = lib.fj_poisson_noalloc(nr, npl, d_ar.data_ptr(), d_rhl.data_ptr(), *[o.data_ptr() for o in outs],
                                    stream)
        assert rc == 0, f"call {call}: fj_poisson_noalloc returned {rc}"
        torch.cuda.synchronize()
        for o, r, name in zip(outs, ref, ("phil", "Pr", "Pr2")):
            assert _shell_rel(o.cpu().numpy(), r) < 1e-9, f"call {call}: {name}"

    big = 2 * 1024 // npl + 1  # nr * npoly above the workspace limit
    rc = lib.fj_poisson_noalloc(big, npl, d_ar.data_ptr(), d_rhl.data_ptr(), *[d_rhl.data_ptr()] * 3, stream)
    assert rc == 1  # FJ_ERR_ARG
