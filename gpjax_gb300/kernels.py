"""Stationary kernels RBF, Matern32, Matern52, Matern12 and RationalQuadratic with ARD lengthscales
(mirrors gpjax/kernels/base.py:42-149 and kernels/stationary/*.py).

Pointwise definitions (on x/l, y/l):
  RBF       s2 exp(-|x-y|^2/2)                          rbf.py:40-44
  Matern32  s2 (1 + sqrt3 t) exp(-sqrt3 t)              matern32.py:41-54
  Matern52  s2 (1 + sqrt5 t + 5/3 t^2) exp(-sqrt5 t)    matern52.py:42-53
  Matern12  s2 exp(-t)                                  matern12.py:44-48
  RationalQuadratic  s2 (1 + |x-y|^2 / (2 alpha))^-alpha  rational_quadratic.py:76-83
with t = sqrt(max(|x-y|^2, 1e-36)) (stationary/utils.py:56-67).
"""
from __future__ import annotations

import torch

from . import _lib
from .computations import AbstractKernelComputation, DenseKernelComputation
from .parameters import NonNegativeReal, PositiveReal


class AbstractKernel:
    name = "AbstractKernel"

    def __init__(self, active_dims=None, n_dims=None,
                 compute_engine: AbstractKernelComputation | None = None):
        self.active_dims = active_dims if active_dims is not None else slice(None)
        self.n_dims = n_dims
        self.compute_engine = compute_engine if compute_engine is not None else \
            DenseKernelComputation()

    def slice_input(self, x: torch.Tensor) -> torch.Tensor:
        """Selects the active input columns (kernels/base.py:137-149)."""
        if isinstance(self.active_dims, slice) and self.active_dims == slice(None):
            return x
        return x[..., self.active_dims]

    def cross_covariance(self, x, y):
        return self.compute_engine.cross_covariance(self, x, y)

    def gram(self, x):
        return self.compute_engine.gram(self, x)

    def diagonal(self, x):
        return self.compute_engine.diagonal(self, x)


class StationaryKernel(AbstractKernel):
    """Stationary kernel with lengthscale [D] or scalar and variance."""

    kind = -1

    def __init__(self, active_dims=None, lengthscale=1.0, variance=1.0, n_dims=None,
                 compute_engine: AbstractKernelComputation | None = None):
        if isinstance(active_dims, (list, tuple)) and n_dims is None:
            n_dims = len(active_dims)
        super().__init__(active_dims, n_dims, compute_engine)
        self.lengthscale = lengthscale if isinstance(lengthscale, PositiveReal) else \
            PositiveReal(lengthscale)
        self.variance = variance if isinstance(variance, NonNegativeReal) else \
            NonNegativeReal(variance)
        ls = self.lengthscale.value
        if ls.ndim > 1:
            raise ValueError("lengthscale must be a scalar or a vector")
        if ls.ndim == 1 and ls.numel() > 1:
            if self.n_dims is not None and self.n_dims != ls.numel():
                raise ValueError("Expected `lengthscale` to be compatible with the number of "
                                 f"input dimensions. Got {ls.numel()} and {self.n_dims}")
            self.n_dims = ls.numel()

    @property
    def n_ls(self) -> int:
        return int(self.lengthscale.value.numel())

    def theta_vector(self, device, obs_stddev=None, constant=None) -> torch.Tensor:
        """[lengthscale..., variance, obs_stddev, constant] as one float64 device vector."""
        z = torch.zeros(1, dtype=torch.float64, device=device)
        parts = [self.lengthscale.value.reshape(-1).to(device),
                 self.variance.value.reshape(1).to(device),
                 z if obs_stddev is None else obs_stddev.reshape(1).to(device),
                 z if constant is None else constant.reshape(1).to(device)]
        return torch.cat(parts)

    def __call__(self, x: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
        """k(x, y) for a pair of points."""
        return self.cross_covariance(x.reshape(1, -1), y.reshape(1, -1))[0, 0]


class RBF(StationaryKernel):
    name = "RBF"
    kind = _lib.RBF


class Matern32(StationaryKernel):
    name = "Matérn32"
    kind = _lib.MATERN32


class Matern52(StationaryKernel):
    name = "Matérn52"
    kind = _lib.MATERN52


class Matern12(StationaryKernel):
    name = "Matérn12"
    kind = _lib.MATERN12


class RationalQuadratic(StationaryKernel):
    """Rational quadratic kernel (kernels/stationary/rational_quadratic.py:40-83).

    ``alpha`` is a fixed shape constant, as in the reference (stored as a plain
    attribute there, not a trainable parameter); it travels to the library in
    one more theta slot after the mean constant."""

    name = "Rational Quadratic"
    kind = _lib.RATIONAL_QUADRATIC

    def __init__(self, active_dims=None, lengthscale=1.0, variance=1.0, alpha=1.0, n_dims=None,
                 compute_engine: AbstractKernelComputation | None = None):
        a = float(alpha.value) if hasattr(alpha, "value") else float(alpha)
        if not a > 0:
            raise ValueError("alpha must be > 0")
        self.alpha = a
        super().__init__(active_dims, lengthscale, variance, n_dims, compute_engine)

    def theta_vector(self, device, obs_stddev=None, constant=None) -> torch.Tensor:
        base = super().theta_vector(device, obs_stddev, constant)
        return torch.cat([base, torch.full((1,), self.alpha, dtype=torch.float64,
                                           device=base.device)])
