"""The tensor-core (tcgen05) BF16 GEMM against torch's FP32 product of the same
BF16 inputs: FP32 accumulation in a different order, so relative 1e-5 of the
largest |C| (K <= 1024)."""
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K,ksplit", [(128, 128, 64, 1), (128, 16, 16, 1), (300, 48, 208, 1),
                                           (1000, 256, 1024, 1), (1000, 256, 1024, 4), (4096, 128, 128, 1)])
def test_tc_gemm(ctx, M, N, K, ksplit):
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    a = torch.randn(M, K, device="cuda", generator=g).bfloat16()
    b = torch.randn(N, K, device="cuda", generator=g).bfloat16()
    c = torch.full((M, N), float("nan"), device="cuda")
    ctx.tc_gemm(a, b, c, ksplit=ksplit)
    ref = a.float() @ b.float().T
    torch.cuda.synchronize()
    err = (c - ref).abs().max().item()
    assert err <= 1e-5 * ref.abs().max().item(), err


def test_tc_gemm_arguments(ctx):
    a = torch.zeros(128, 24, device="cuda").bfloat16()  # K not a multiple of 16
    b = torch.zeros(16, 24, device="cuda").bfloat16()
    c = torch.zeros(128, 16, device="cuda")
    import fjmodels_gb300 as F
    with pytest.raises(F.FJError):
        ctx.tc_gemm(a, b, c)
