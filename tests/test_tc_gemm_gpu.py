"""GPU: the tcgen05 split-TF32 GEMM (gpk_gemm_tf32x3) against a float64
product of the same float32 inputs.  Tolerance: 2e-5 of |A| |B|^T elementwise
(float32 accumulation over K with TF32x3 products)."""
import numpy as np
import pytest
import torch

from gpjax_gb300 import _lib

pytestmark = pytest.mark.gpu


def gemm(A, B, C, alpha=1.0, beta=0.0, lower=False):
    M, K = A.shape
    N = B.shape[0]
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    nbytes = _lib.lib().gpk_gemm_tf32x3_workspace_bytes(M, N, K)
    ws = _lib.workspace(nbytes, A.device)
    _lib.call("gpk_gemm_tf32x3", M, N, K, alpha, A.data_ptr(), A.stride(0), B.data_ptr(),
              B.stride(0), beta, C.data_ptr(), C.stride(0), int(lower), err.data_ptr(),
              ws.data_ptr(), ws.numel(), _lib.stream_ptr(A.device))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return C


# sizes from 2048 up use the 128 x 256 tile (ragged edges included)
@pytest.mark.parametrize("M,N,K", [(128, 128, 128), (256, 384, 96), (1000, 777, 513),
                                   (129, 130, 31), (2048, 2048, 2048), (64, 512, 4096),
                                   (2176, 2304, 1000), (2300, 2050, 77)])
def test_split_tf32_gemm(cuda_lib, M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g)
    B = torch.randn(N, K, device="cuda", generator=g)
    C = torch.randn(M, N, device="cuda", generator=g)
    C0 = C.clone()
    gemm(A, B, C, alpha=-1.0, beta=1.0)
    ref = C0.double() - A.double() @ B.double().T
    bound = A.double().abs() @ B.double().abs().T
    err = (C.double() - ref).abs()
    assert bool(torch.all(err <= 2e-5 * bound + 1e-6)), float((err / (bound + 1e-30)).max())


@pytest.mark.parametrize("n,K", [(640, 256), (2304, 512), (2200, 96)])
def test_split_tf32_gemm_lower_only(cuda_lib, n, K):
    g = torch.Generator(device="cuda").manual_seed(7 + n)
    P = torch.randn(n, K, device="cuda", generator=g)
    C = torch.zeros(n, n, device="cuda")
    gemm(P, P, C, alpha=1.0, beta=0.0, lower=True)
    ref = (P.double() @ P.double().T)
    low = torch.tril(torch.ones(n, n, dtype=torch.bool, device="cuda"))
    assert bool(torch.all(C[~low] == 0))
    bound = P.double().abs() @ P.double().abs().T
    assert bool(torch.all(((C.double() - ref).abs() <= 2e-5 * bound + 1e-6)[low]))


def test_split_tf32_beats_plain_tf32_accuracy(cuda_lib):
    # the split recovers near-float32 accuracy, two orders below TF32's 2^-11
    # relative rounding (the tensor-core float32 accumulation sets the floor)
    M = N = K = 1024
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn(M, K, device="cuda", generator=g)
    B = torch.randn(N, K, device="cuda", generator=g)
    C = torch.zeros(M, N, device="cuda")
    gemm(A, B, C)
    ref = A.double() @ B.double().T
    rel = float(((C.double() - ref).norm() / ref.norm()))
    print(f"split-TF32 GEMM relative error (K={K}): {rel:.3e}")
    assert rel < 2e-5, rel


def test_split_tf32_cancellation_probe(cuda_lib):
    """A product with heavy cancellation (A times the inverse of a triangular
    factor, as in a triangular solve by multiplication): split-TF32 error
    against float64, with float32 cuBLAS printed beside it."""
    n = 1024
    g = torch.Generator(device="cuda").manual_seed(11)
    X = torch.randn(n, 4, device="cuda", dtype=torch.float64, generator=g)
    K = torch.exp(-0.5 * torch.cdist(X, X) ** 2) + 1e-2 * torch.eye(n, device="cuda",
                                                                      dtype=torch.float64)
    L = torch.linalg.cholesky(K[:512, :512])
    Minv = torch.linalg.inv(L)
    A = K[512:, :512]
    ref = A @ Minv.T
    A32, M32 = A.float().contiguous(), Minv.float().contiguous()
    C = torch.zeros(512, 512, device="cuda")
    gemm(A32, M32, C)
    e_tc = float((C.double() - ref).norm() / ref.norm())
    torch.backends.cuda.matmul.allow_tf32 = False
    e_f32 = float(((A32 @ M32.T).double() - ref).norm() / ref.norm())
    print(f"cancellation probe: split-TF32 {e_tc:.3e}  float32 cuBLAS {e_f32:.3e}")
    assert e_tc < 50 * e_f32 + 1e-6


def test_bounded_wait_runs_out_and_reports(cuda_lib):
    """A device wait that can never be satisfied (the self-test's barrier that
    nothing arrives at) gives up after its bound, reports through the error
    flag and leaves the context usable: a normal GEMM right after it is exact."""
    lib = _lib.lib()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = _lib.workspace(lib.gpk_selftest_wait_timeout_workspace_bytes(), torch.device("cuda"))
    _lib.call("gpk_selftest_wait_timeout", err.data_ptr(), ws.data_ptr(), ws.numel(),
              _lib.stream_ptr())
    torch.cuda.synchronize()
    assert int(err.item()) == 1
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(256, 128, device="cuda", generator=g)
    B = torch.randn(192, 128, device="cuda", generator=g)
    C = torch.zeros(256, 192, device="cuda")
    gemm(A, B, C)
    ref = A.double() @ B.double().T
    assert float((C.double() - ref).abs().max()) <= 2e-5 * float(
        (A.double().abs() @ B.double().abs().T).max())
