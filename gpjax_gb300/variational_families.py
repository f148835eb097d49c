"""Collapsed variational family for SGPR (mirrors
gpjax/variational_families.py:107-131 and 767-870)."""
from __future__ import annotations

import torch

from .distributions import GaussianDistribution
from .likelihoods import Gaussian
from .linalg import Dense, add_jitter, cholesky_dense, psd, solve_triangular
from .parameters import Real


class AbstractVariationalGaussian:
    def __init__(self, posterior, inducing_inputs, jitter: float = 1e-6):
        self.posterior = posterior
        self.inducing_inputs = inducing_inputs if isinstance(inducing_inputs, Real) else \
            Real(inducing_inputs)
        self.jitter = jitter

    @property
    def num_inducing(self) -> int:
        return int(self.inducing_inputs.value.shape[0])


class CollapsedVariationalGaussian(AbstractVariationalGaussian):
    """Titsias' collapsed variational family (variational_families.py:767-784)."""

    def __init__(self, posterior, inducing_inputs, jitter: float = 1e-6):
        super().__init__(posterior, inducing_inputs, jitter)
        if not isinstance(posterior.likelihood, Gaussian):
            raise TypeError("Likelihood must be Gaussian.")

    def predict(self, test_inputs: torch.Tensor, train_data) -> GaussianDistribution:
        """SGPR predictive distribution (variational_families.py:786-870), composed
        from the library's GPU cross-covariance, Cholesky and triangular solves."""
        with torch.no_grad():
            t = test_inputs.to(train_data.X.device, torch.float64)
            x, y = train_data.X, train_data.y
            kernel = self.posterior.prior.kernel
            mean_function = self.posterior.prior.mean_function
            sd = self.posterior.likelihood.obs_stddev.value.to(x.device).detach()
            noise_var = sd**2
            z = self.inducing_inputs.value.to(x.device).detach()
            m = z.shape[0]
            Kzx = kernel.cross_covariance(z, x).detach()
            Kzz = add_jitter(kernel.gram(z).to_dense().detach(), self.jitter)
            Lz, _ = cholesky_dense(Kzz, check=True)
            Lz_inv_Kzx = solve_triangular(Lz, Kzx)
            A = Lz_inv_Kzx / sd
            AAT = A @ A.T
            L, _ = cholesky_dense(torch.eye(m, dtype=torch.float64, device=x.device) + AAT,
                                  check=True)
            diff = y - mean_function(x)
            tmp = solve_triangular(L, Lz_inv_Kzx @ diff)
            Lz_inv_Kzx_diff = solve_triangular(L.T.contiguous(), tmp, lower=False)
            Kzz_inv_Kzx_diff = solve_triangular(Lz.T.contiguous(), Lz_inv_Kzx_diff, lower=False)
            Ktt = kernel.gram(t).to_dense().detach()
            Kzt = kernel.cross_covariance(z, t).detach()
            mut = mean_function(t)
            Lz_inv_Kzt = solve_triangular(Lz, Kzt)
            L_inv_Lz_inv_Kzt = solve_triangular(L, Lz_inv_Kzt)
            mean = mut + (Kzt.T / noise_var) @ Kzz_inv_Kzx_diff
            cov = Ktt - Lz_inv_Kzt.T @ Lz_inv_Kzt + L_inv_Lz_inv_Kzt.T @ L_inv_Lz_inv_Kzt
            cov = add_jitter(cov, self.jitter)
        return GaussianDistribution(mean.reshape(-1), psd(Dense(cov)))
