"""Collapsed variational family for SGPR (mirrors
gpjax/variational_families.py:107-131 and 767-870)."""
from __future__ import annotations

import torch

from .distributions import GaussianDistribution
from .likelihoods import Gaussian
from .linalg import Dense, add_jitter, cholesky_dense, matmul, psd, solve_triangular
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
        """SGPR predictive distribution (variational_families.py:786-870): every
        product and solve is a library call -- cross-covariances and Grams,
        Cholesky factors, triangular solves (including the transposed ones the
        reference makes with cho_solve and solve_triangular(L.T)) and float64
        GEMMs; torch only holds the tensors."""
        with torch.no_grad():
            t = test_inputs.to(train_data.X.device, torch.float64)
            x, y = train_data.X, train_data.y
            kernel = self.posterior.prior.kernel
            mean_function = self.posterior.prior.mean_function
            sd = float(self.posterior.likelihood.obs_stddev.value)
            noise_var = sd * sd
            z = self.inducing_inputs.value.to(x.device).detach()
            Kzx = kernel.cross_covariance(z, x).detach()                       # :815
            Kzz = add_jitter(kernel.gram(z).to_dense().detach(), self.jitter)   # :816-818
            Lz, _ = cholesky_dense(Kzz, check=True)                             # :821
            Lz_inv_Kzx = solve_triangular(Lz, Kzx)                              # :824
            AAT = matmul(Lz_inv_Kzx, Lz_inv_Kzx, transb=True, alpha=1.0 / noise_var)  # :827-830
            L, _ = cholesky_dense(add_jitter(AAT, 1.0), check=True)             # :833
            diff = (y - mean_function(x)).reshape(-1, 1)                        # :835-836
            v = matmul(Lz_inv_Kzx, diff)
            v = solve_triangular(L, solve_triangular(L, v), trans=True)         # cho_solve :839
            w = solve_triangular(Lz, v, trans=True)                             # Lz^-T :842
            Ktt = kernel.gram(t).to_dense().detach()                            # :844
            Kzt = kernel.cross_covariance(z, t).detach()                        # :845
            Ktz = kernel.cross_covariance(t, z).detach()                        # Kzt^T
            mut = mean_function(t)                                              # :846
            Q = solve_triangular(Lz, Kzt)                                       # :849
            R = solve_triangular(L, Q)                                          # :852
            mean = mut.reshape(-1, 1) + matmul(Ktz, w, alpha=1.0 / noise_var)    # :855
            cov = Ktt - matmul(Q, Q, transa=True) + matmul(R, R, transa=True)   # :858-862
            cov = add_jitter(cov, self.jitter)                                  # :865
        return GaussianDistribution(mean.reshape(-1), psd(Dense(cov)))
