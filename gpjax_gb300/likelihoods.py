"""Gaussian likelihood (mirrors gpjax/likelihoods.py:129-187)."""
from __future__ import annotations

import torch

from .parameters import NonNegativeReal


class Gaussian:
    """y = f + e, e ~ N(0, obs_stddev^2)."""

    def __init__(self, num_datapoints: int, obs_stddev=1.0):
        self.num_datapoints = num_datapoints
        self.obs_stddev = obs_stddev if isinstance(obs_stddev, NonNegativeReal) else \
            NonNegativeReal(obs_stddev)

    def predict(self, dist):
        """Adds obs_stddev^2 to the covariance diagonal (likelihoods.py:165-187)."""
        from .distributions import GaussianDistribution
        from .linalg import Dense
        cov = dist.covariance().clone()
        idx = torch.arange(cov.shape[0], device=cov.device)
        cov[idx, idx] += self.obs_stddev.value.to(cov.device) ** 2
        return GaussianDistribution(dist.mean, Dense(cov))
