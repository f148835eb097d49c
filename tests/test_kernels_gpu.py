"""GPU parity of Gram / cross-covariance / diagonal and of the linear-algebra
operations against the float64 oracle and numpy."""
import numpy as np
import pytest
import torch

import gpjax_gb300 as gpx
from gpjax_gb300 import kernels as K
from gpjax_gb300 import linalg as LA
from oracle import gp_oracle as O

pytestmark = pytest.mark.gpu


def _kern(cls, ls, var):
    if cls is K.RationalQuadratic:
        return cls(lengthscale=ls, variance=var, alpha=0.7)
    return cls(lengthscale=ls, variance=var)


@pytest.mark.parametrize("cls,kind", [(K.RBF, O.RBF), (K.Matern32, O.MATERN32),
                                      (K.Matern52, O.MATERN52), (K.Matern12, O.MATERN12),
                                      (K.RationalQuadratic, O.rational_quadratic(0.7))])
@pytest.mark.parametrize("n,m,d", [(1, 1, 1), (7, 3, 2), (65, 130, 8), (200, 33, 16)])
def test_cross_covariance_parity(cuda_lib, cls, kind, n, m, d):
    rng = np.random.default_rng(n + m + d)
    x, y = rng.standard_normal((n, d)), rng.standard_normal((m, d))
    ls = np.exp(rng.uniform(-1, 1, d))
    k = _kern(cls, ls, 0.7)
    out = k.cross_covariance(torch.as_tensor(x, device="cuda"),
                             torch.as_tensor(y, device="cuda")).cpu().numpy()
    ref = O.cross_covariance(kind, x, y, ls, 0.7)
    assert np.allclose(out, ref, rtol=1e-13, atol=1e-14)
    G = k.gram(torch.as_tensor(x, device="cuda")).to_dense().cpu().numpy()
    assert np.allclose(G, O.gram(kind, x, ls, 0.7), rtol=1e-13, atol=1e-14)
    dg = k.diagonal(torch.as_tensor(x, device="cuda")).diagonal.cpu().numpy()
    assert np.allclose(dg, O.diagonal(kind, x, ls, 0.7))


def test_compute_engine_swap_keeps_diagonal(cuda_lib):
    # tests/test_kernels/test_computation.py:43-81 of the reference
    x = torch.randn(20, 3, dtype=torch.float64, device="cuda")
    k = K.RBF(lengthscale=np.array([0.5, 1.0, 2.0]), variance=1.5)
    d1 = torch.diagonal(k.gram(x).to_dense())
    k.compute_engine = gpx.computations.DiagonalKernelComputation()
    d2 = k.gram(x).diagonal
    assert torch.allclose(d1, d2)


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-11), (torch.float32, 2e-4)])
@pytest.mark.parametrize("n", [1, 2, 3, 64, 65, 127, 128, 129, 300, 700])
def test_cholesky_solve_logdet(cuda_lib, dtype, tol, n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    A = A @ A.T / n + np.eye(n)
    At = torch.as_tensor(A, device="cuda", dtype=dtype)
    L = LA.lower_cholesky(LA.Dense(At)).to_dense().double().cpu().numpy()
    Lref = np.linalg.cholesky(A)
    assert np.allclose(L, Lref, rtol=tol, atol=tol)
    B = rng.standard_normal((n, 5))
    X = LA.solve(LA.Triangular(torch.as_tensor(Lref, device="cuda", dtype=dtype)),
                 torch.as_tensor(B, device="cuda", dtype=dtype)).double().cpu().numpy()
    assert np.allclose(Lref @ X, B, rtol=tol * 10, atol=tol * 10)
    ld = float(LA.logdet(LA.Dense(At)))
    assert np.isclose(ld, np.linalg.slogdet(A)[1], rtol=tol, atol=tol * n)


def test_linalg_known_answers(cuda_lib):
    # tests/test_linalg.py:237-396 of the reference
    A = torch.tensor([[2.0, 1.0], [1.0, 3.0]], dtype=torch.float64, device="cuda")
    b = torch.tensor([1.0, 2.0], dtype=torch.float64, device="cuda")
    x = LA.solve(LA.Dense(A), b)
    assert torch.allclose(A @ x, b)
    assert np.isclose(float(LA.logdet(LA.Dense(A))), np.log(5.0))
    L = torch.tensor([[2.0, 0.0], [1.0, 3.0]], dtype=torch.float64, device="cuda")
    xt = LA.solve(LA.Triangular(L), torch.tensor([2.0, 7.0], dtype=torch.float64, device="cuda"))
    assert torch.allclose(L @ xt, torch.tensor([2.0, 7.0], dtype=torch.float64, device="cuda"))
    assert np.isclose(float(LA.logdet(LA.Triangular(L))), np.log(6.0))


def test_cholesky_not_pd_reports_info(cuda_lib):
    A = torch.tensor([[1.0, 2.0], [2.0, 1.0]], dtype=torch.float64, device="cuda")
    L, info = LA.cholesky_dense(A)
    assert int(info.item()) == 2
    assert torch.isnan(L[1, 1])


@pytest.mark.parametrize("cls,kind", [(K.Matern12, O.MATERN12),
                                      (K.RationalQuadratic, O.rational_quadratic(0.7))])
def test_cross_covariance_vjp_added_kernels(cuda_lib, cls, kind):
    """Gradient of sum(G * K(x, y)) w.r.t. lengthscales, variance and both inputs
    against torch float64 autograd of the oracle's kernel."""
    rng = np.random.default_rng(3)
    x, y = rng.standard_normal((40, 3)), rng.standard_normal((25, 3))
    ls = np.exp(rng.uniform(-0.5, 0.5, 3))
    G = rng.standard_normal((40, 25))
    k = _kern(cls, ls, 0.9)
    k.lengthscale.to("cuda").requires_grad_(True)
    k.variance.to("cuda").requires_grad_(True)
    X = torch.as_tensor(x, device="cuda").requires_grad_(True)
    Y = torch.as_tensor(y, device="cuda").requires_grad_(True)
    (k.cross_covariance(X, Y) * torch.as_tensor(G, device="cuda")).sum().backward()
    lt = torch.tensor(ls, requires_grad=True)
    vt = torch.tensor(0.9, dtype=torch.float64, requires_grad=True)
    xt = torch.tensor(x, requires_grad=True)
    yt = torch.tensor(y, requires_grad=True)
    (O._t_kernel(kind, xt, yt, lt, vt) * torch.as_tensor(G)).sum().backward()
    for got, ref in ((k.lengthscale.value.grad, lt.grad), (k.variance.value.grad, vt.grad),
                     (X.grad, xt.grad), (Y.grad, yt.grad)):
        assert np.allclose(got.cpu().numpy(), ref.numpy(), rtol=1e-9, atol=1e-11)


@pytest.mark.parametrize("upper", [False, True])
@pytest.mark.parametrize("trans", [False, True])
@pytest.mark.parametrize("n,k", [(1, 1), (65, 3), (300, 40)])
def test_triangular_solve_variants(cuda_lib, upper, trans, n, k):
    """op(T) X = B for lower / upper T and op = identity / transpose
    (jax.scipy.linalg.solve_triangular's lower and trans flags)."""
    rng = np.random.default_rng(n + k)
    T = np.tril(rng.standard_normal((n, n))) + n * np.eye(n)
    if upper:
        T = T.T.copy()
    B = rng.standard_normal((n, k))
    X = LA.solve_triangular(torch.as_tensor(T, device="cuda"), torch.as_tensor(B, device="cuda"),
                            lower=not upper, trans=trans).cpu().numpy()
    ref = np.linalg.solve(T.T if trans else T, B)
    assert np.allclose(X, ref, rtol=1e-11, atol=1e-12)


@pytest.mark.parametrize("transa", [False, True])
@pytest.mark.parametrize("transb", [False, True])
@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (70, 33, 129), (256, 300, 64)])
def test_gemm_f64(cuda_lib, transa, transb, m, n, k):
    rng = np.random.default_rng(m * n + k)
    A = rng.standard_normal((k, m) if transa else (m, k))
    B = rng.standard_normal((n, k) if transb else (k, n))
    C = LA.matmul(torch.as_tensor(A, device="cuda"), torch.as_tensor(B, device="cuda"),
                  transa=transa, transb=transb, alpha=0.5).cpu().numpy()
    ref = 0.5 * (A.T if transa else A) @ (B.T if transb else B)
    assert np.allclose(C, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
