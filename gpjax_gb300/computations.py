"""Kernel compute engines (mirrors gpjax/kernels/computations/base.py:36-109 and
dense.py:23-36).  ``DenseKernelComputation`` evaluates cross-covariances,
Gram matrices and diagonals on the GPU through libgpk.so; the engine is
swappable at runtime exactly like the reference's ``compute_engine``
attribute (tests/test_kernels/test_computation.py:29-81).
"""
from __future__ import annotations

import torch

from . import _lib
from .linalg import Dense, Diagonal, psd


class _CrossCov(torch.autograd.Function):
    """K(x, y) with gradients w.r.t. the kernel hyperparameters and the inputs."""

    @staticmethod
    def forward(ctx, theta, x, y, kind, n_ls, out_dtype):
        dev = _lib.require_cuda(x, y, theta)
        n, m, d = x.shape[0], y.shape[0], x.shape[1]
        code = _lib.F64 if out_dtype == torch.float64 else _lib.F32
        out = torch.empty((n, m), dtype=out_dtype, device=dev)
        xc, yc, th = x.detach().contiguous(), y.detach().contiguous(), theta.detach().contiguous()
        _lib.call("gpk_cross_covariance", kind, n, m, d, xc.data_ptr(), d, yc.data_ptr(), d,
                  th.data_ptr(), n_ls, code, out.data_ptr(), m, _lib.stream_ptr(dev))
        ctx.save_for_backward(th, xc, yc)
        ctx.kind, ctx.n_ls = kind, n_ls
        return out

    @staticmethod
    def backward(ctx, g):
        th, xc, yc = ctx.saved_tensors
        from .objectives import cross_covariance_vjp
        gth, gx, gy = cross_covariance_vjp(ctx.kind, ctx.n_ls, th, xc, yc, g.to(torch.float64),
                                           need_x=ctx.needs_input_grad[1],
                                           need_y=ctx.needs_input_grad[2])
        return gth, gx, gy, None, None, None


class AbstractKernelComputation:
    """Computes Gram, cross-covariance and diagonal of a kernel."""

    def _cross_covariance(self, kernel, x, y):  # pragma: no cover - interface
        raise NotImplementedError

    def cross_covariance(self, kernel, x: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
        """[N, M] cross-covariance (computations/base.py:79-93)."""
        return self._cross_covariance(kernel, x, y)

    def gram(self, kernel, x: torch.Tensor) -> Dense:
        """psd(Dense(K(x, x))) (computations/base.py:56-72)."""
        return psd(Dense(self.cross_covariance(kernel, x, x)))

    def _diagonal(self, kernel, inputs: torch.Tensor) -> Diagonal:
        xs = kernel.slice_input(inputs)
        dev = _lib.require_cuda(xs)
        th = kernel.theta_vector(dev).detach().contiguous()
        out = torch.empty(xs.shape[0], dtype=torch.float64, device=dev)
        xc = xs.detach().contiguous()
        _lib.call("gpk_diagonal", kernel.kind, xc.shape[0], xc.shape[1], xc.data_ptr(),
                  xc.shape[1], th.data_ptr(), kernel.n_ls, out.data_ptr(), _lib.stream_ptr(dev))
        return psd(Diagonal(out))

    def diagonal(self, kernel, inputs: torch.Tensor) -> Diagonal:
        """diag k(x_i, x_i) (computations/base.py:95-109)."""
        return self._diagonal(kernel, inputs)


class DenseKernelComputation(AbstractKernelComputation):
    """Dense evaluation on the GPU (computations/dense.py:23-36)."""

    def __init__(self, out_dtype: torch.dtype = torch.float64):
        self.out_dtype = out_dtype

    def _cross_covariance(self, kernel, x, y):
        xs, ys = kernel.slice_input(x), kernel.slice_input(y)
        dev = _lib.require_cuda(xs, ys)
        th = kernel.theta_vector(dev)
        return _CrossCov.apply(th, xs, ys, kernel.kind, kernel.n_ls, self.out_dtype)


class DiagonalKernelComputation(AbstractKernelComputation):
    """Diagonal-only Gram (computations/diagonal.py:33-46)."""

    def gram(self, kernel, x):
        return self.diagonal(kernel, x)

    def _cross_covariance(self, kernel, x, y):
        return DenseKernelComputation()._cross_covariance(kernel, x, y)
