"""The tcgen05 BF16 GEMM of the learned surrogate, C = A Bt^T (+ bias),
through the C ABI on torch-allocated device buffers.  Integer-valued
operands keep every product and partial sum exact in fp32, so the tensor-core
result must equal the fp32 reference exactly whatever the summation order."""
import ctypes as C

import pytest

torch = pytest.importorskip("torch")
from eprem_gb300.runtime import load_library  # noqa: E402

pytestmark = pytest.mark.gpu


def _gemm(A, Bt, bias=None):
    lib = load_library()
    M, K = A.shape
    N = Bt.shape[0]
    out = torch.full((M, N), float("nan"), device="cuda", dtype=torch.float32)
    rc = lib.eprem_gpu_gemm_bf16(A.data_ptr(), A.stride(0), Bt.data_ptr(), Bt.stride(0),
                                 bias.data_ptr() if bias is not None else None, out.data_ptr(),
                                 out.stride(0), M, N, K, None)
    assert rc == 0, lib.eprem_gpu_last_error().decode()
    return out


def _ints(shape, lo=-4, hi=5, seed=0):
    g = torch.Generator().manual_seed(seed)
    return torch.randint(lo, hi, shape, generator=g).to(torch.bfloat16).cuda()


def test_single_mma_tile():
    A = _ints((128, 16), seed=1)
    Bt = _ints((16, 16), seed=2)
    ref = A.float() @ Bt.float().T
    torch.testing.assert_close(_gemm(A, Bt), ref, rtol=0, atol=0)


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (300, 48, 256), (4096, 256, 48),
                                   (256, 48, 8192), (130, 40, 24)])
def test_gemm_shapes(M, N, K):
    A = _ints((M, K), seed=M + K)
    Bt = _ints((N, K), seed=N + 7)
    bias = torch.arange(N, dtype=torch.float32, device="cuda") * 0.5
    ref = A.float() @ Bt.float().T + bias
    torch.testing.assert_close(_gemm(A, Bt, bias), ref, rtol=0, atol=0)


def test_gemm_real_values_within_fp32_rounding():
    g = torch.Generator().manual_seed(3)
    A = torch.randn((512, 256), generator=g).to(torch.bfloat16).cuda()
    Bt = torch.randn((256, 256), generator=g).to(torch.bfloat16).cuda()
    ref = A.double() @ Bt.double().T
    got = _gemm(A, Bt).double()
    assert float((got - ref).abs().max() / ref.abs().max()) < 1e-5
