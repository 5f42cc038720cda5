"""fj_poisson_noalloc: the Poisson solve without a context, for callers that hold
no fj_ctx or cannot allocate device memory on their call path (their device memory
belongs to their own pool allocator, or the call sits in a latency-bound loop).
The Poisson kernel keeps its quadrature workspace in shared memory, so the entry
point needs only its inputs, outputs and a stream.  This file is collected last so
that a failure here leaves every other test already run; it passes on its own in a
fresh process too.

Checked through the C ABI: two calls in a row give the same tables as fj_poisson
(the same kernel: equal bits), so does a grid of more than a thousand coefficients,
and bad arguments are refused with FJ_ERR_ARG before any GPU work.  In a fresh
process that never made a context, the calls leave the device's per-thread stack
limit as they found it (a kernel whose stack exceeded it would make the driver
grow the local-memory reservation: the one allocation a launch can make).
"""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fjmodels_gb300 as F  # noqa: E402

pytestmark = pytest.mark.gpu


def _case(nr, npl, seed):
    ar = F.log_grid(1e-3, 300.0, nr)
    rhl = F.guess_rhl(ar, 40, npl, "NFW")
    rng = np.random.default_rng(seed)  # a non-spherical density: seeded multipoles l > 0
    rhl[1:, 1:] = rhl[1:, :1] * rng.uniform(-0.05, 0.05, size=(nr - 1, npl - 1))
    f64 = dict(dtype=torch.float64, device="cuda")
    return torch.tensor(ar, **f64), torch.tensor(rhl, **f64)


def _context_poisson(d_ar, d_rhl):
    nr, npl = d_rhl.shape
    ctx = F.Context(0)
    ref = [torch.zeros((nr, npl), dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.computePhil(d_ar, d_rhl, *ref)
    torch.cuda.synchronize()
    ctx.close()
    return [t.cpu().numpy() for t in ref]


def _noalloc(lib, d_ar, d_rhl, stream):
    nr, npl = d_rhl.shape
    outs = [torch.full((nr, npl), np.nan, dtype=torch.float64, device="cuda") for _ in range(3)]
    rc = lib.fj_poisson_noalloc(nr, npl, d_ar.data_ptr(), d_rhl.data_ptr(), *[o.data_ptr() for o in outs], stream)
    torch.cuda.synchronize()
    return rc, [o.cpu().numpy() for o in outs]


def test_noalloc_poisson_matches_context_poisson():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = F.load_library()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for nr, npl in ((80, 7), (200, 7)):  # 560 and 1400 coefficients
        d_ar, d_rhl = _case(nr, npl, 7)
        ref = _context_poisson(d_ar, d_rhl)
        for call in range(2):
            rc, outs = _noalloc(lib, d_ar, d_rhl, stream)
            assert rc == 0, f"{nr} x {npl}, call {call}: fj_poisson_noalloc returned {rc}"
            for o, r, name in zip(outs, ref, ("phil", "Pr", "Pr2")):
                assert np.array_equal(o, r), f"{nr} x {npl}, call {call}: {name}"
    d_ar, d_rhl = _case(80, 7, 7)
    for bad in ((1, 7), (80, 0), (80, 64)):
        rc = lib.fj_poisson_noalloc(*bad, d_ar.data_ptr(), d_rhl.data_ptr(), *[d_rhl.data_ptr()] * 3, stream)
        assert rc == 1, bad  # FJ_ERR_ARG


FRESH = r"""
import ctypes as C, json, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
import fjmodels_gb300 as F
lib = F.load_library()
need, lim0, lim1 = C.c_size_t(), C.c_size_t(), C.c_size_t()
assert lib.fj_poisson_noalloc_stack(C.byref(need), C.byref(lim0)) == 0
nr, npl = 80, 7
ar = F.log_grid(1e-3, 300.0, nr)
rhl = F.guess_rhl(ar, 40, npl, "NFW")
f64 = dict(dtype=torch.float64, device="cuda")
d_ar, d_rhl = torch.tensor(ar, **f64), torch.tensor(rhl, **f64)
outs = [[torch.zeros((nr, npl), **f64) for _ in range(3)] for _ in range(2)]
s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
rcs = [lib.fj_poisson_noalloc(nr, npl, d_ar.data_ptr(), d_rhl.data_ptr(), *[o.data_ptr() for o in oo], s)
       for oo in outs]
torch.cuda.synchronize()
assert lib.fj_poisson_noalloc_stack(None, C.byref(lim1)) == 0
ctx = F.Context(0)
ref = [torch.zeros((nr, npl), **f64) for _ in range(3)]
ctx.computePhil(d_ar, d_rhl, *ref)
torch.cuda.synchronize()
same = all(torch.equal(o, r) for oo in outs for o, r in zip(oo, ref))
ctx.close()
print(json.dumps({"rc": rcs, "need": need.value, "limit_before": lim0.value, "limit_after": lim1.value,
                  "same": same}))
"""


def test_noalloc_fresh_process_keeps_stack_limit():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", FRESH, root], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["rc"] == [0, 0], out
    assert out["need"] <= out["limit_before"], out
    assert out["limit_after"] == out["limit_before"], out
    assert out["same"], out
