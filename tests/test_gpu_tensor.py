"""The tcgen05 BF16 GEMM against an FP32 matmul of the same BF16 operands."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (128, 256, 64), (256, 128, 192), (384, 320, 128), (128, 512, 1024)])
def test_gemm_matches_fp32(M, N, K):
    from piqmc.tensor import gemm_bf16
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    D = gemm_bf16(A, B)
    ref = A.double() @ B.double().T
    err = (D.double() - ref).abs().max().item()
    # FP32 accumulation of K products of BF16 values (exact products): error ~ K * 2^-24 * max|partial sum|
    assert err <= 1e-5 * K ** 0.5 * ref.abs().max().item() + 1e-4, err


def test_gemm_alpha_bias_and_signs():
    from piqmc.tensor import gemm_bf16
    M, N, K = 256, 128, 128
    A = torch.where(torch.rand(M, K, device="cuda") < 0.5, -1.0, 1.0).to(torch.bfloat16)   # spins are exact in BF16
    B = torch.randint(-4, 5, (N, K), device="cuda").to(torch.bfloat16)
    bias = torch.randn(N, device="cuda")
    D = gemm_bf16(A, B, alpha=0.5, bias=bias)
    ref = 0.5 * (A.float() @ B.float().T) + bias
    assert torch.allclose(D, ref, atol=1e-5, rtol=0)
