"""GaussianDistribution (mirrors gpjax/distributions.py:42-134)."""
from __future__ import annotations

import math

import torch

from .linalg import LinearOperator, diag, logdet, psd, solve


class GaussianDistribution:
    """Multivariate normal with mean ``loc`` [n] and covariance operator ``scale``."""

    def __init__(self, loc: torch.Tensor, scale: LinearOperator | None):
        self.loc = loc
        self.scale = psd(scale) if scale is not None else None
        self._variance = None

    @property
    def mean(self) -> torch.Tensor:
        return self.loc

    @property
    def event_shape(self):
        return tuple(self.loc.shape)

    @property
    def variance(self) -> torch.Tensor:
        """diag(cov) (distributions.py:79-81)."""
        if self._variance is not None:
            return self._variance
        return diag(self.scale)

    def stddev(self) -> torch.Tensor:
        return torch.sqrt(self.variance)

    def covariance(self) -> torch.Tensor:
        return self.scale.to_dense()

    @property
    def covariance_matrix(self) -> torch.Tensor:
        return self.covariance()

    def entropy(self) -> torch.Tensor:
        return 0.5 * (self.loc.shape[0] * (1.0 + math.log(2.0 * math.pi)) + logdet(self.scale))

    def log_prob(self, y: torch.Tensor) -> torch.Tensor:
        """-1/2 (n log 2pi + log|S| + diff^T S^-1 diff) (distributions.py:115-134)."""
        diff = y - self.loc
        n = self.loc.shape[-1]
        return -0.5 * (n * math.log(2.0 * math.pi) + logdet(self.scale) +
                       diff @ solve(self.scale, diff))
