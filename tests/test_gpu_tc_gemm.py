"""The tensor-core contraction of the surrogate (tc_gemm.cu) against a
plain PyTorch FP32 reference of the same op on the same BF16 inputs.

Tolerance: BF16 products are exact in FP32, so only the FP32 summation
order differs: max |D - ref| <= 1e-5 * (sum_k |A||B| max) per case; BF16
outputs add their own rounding (relative 2^-8)."""
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _ref(A, B, bias=None, act=0, Dadd=None):
    r = A.float() @ B.float().T
    if bias is not None:
        r = r + bias
    if Dadd is not None:
        r = r + Dadd
    if act == 1:
        r = torch.nn.functional.gelu(r, approximate="tanh")
    return r


def _scale(A, B):
    return (A.float().abs() @ B.float().abs().T).max().item()


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (128, 32, 64), (300, 100, 200), (1000, 32, 32),
                                   (4096, 128, 1024), (257, 64, 8), (129, 48, 520)])
def test_tc_gemm_fp32(lib, M, N, K):
    import hosnwt
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    D = hosnwt.tc_gemm(A, B, err=err)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = _ref(A, B)
    assert (D - ref).abs().max().item() <= 1e-5 * _scale(A, B)


def test_tc_gemm_epilogue(lib):
    import hosnwt
    g = torch.Generator(device="cuda").manual_seed(3)
    M, N, K = 700, 96, 160
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    Dadd = torch.randn(M, N, device="cuda", generator=g)
    D = hosnwt.tc_gemm(A, B, bias=bias, act=1, Dadd=Dadd)
    ref = _ref(A, B, bias, 1, Dadd)
    assert (D - ref).abs().max().item() <= 1e-5 * _scale(A, B) + 1e-5
    Db = hosnwt.tc_gemm(A, B, bias=bias, act=0, out_bf16=True)
    refb = _ref(A, B, bias)
    assert ((Db.float() - refb).abs() <= 2.0 ** -7 * refb.abs() + 1e-5 * _scale(A, B)).all()


def test_tc_gemm_strided_operands(lib):
    """Operands that are row slices of wider matrices (row strides > K)."""
    import hosnwt
    g = torch.Generator(device="cuda").manual_seed(5)
    Aw = torch.randn(256, 136, device="cuda", generator=g).to(torch.bfloat16)
    Bw = torch.randn(64, 200, device="cuda", generator=g).to(torch.bfloat16)
    A, B = Aw[:, :128], Bw[:, :128]
    D = hosnwt.tc_gemm(A, B)
    assert (D - _ref(A, B)).abs().max().item() <= 1e-5 * _scale(A, B)


def test_tc_gemm_rejects_bad_shapes(lib):
    import hosnwt
    A = torch.zeros(16, 12, device="cuda", dtype=torch.bfloat16)  # K not a multiple of 8
    B = torch.zeros(16, 12, device="cuda", dtype=torch.bfloat16)
    with pytest.raises(hosnwt.HosError):
        hosnwt.tc_gemm(A, B)
