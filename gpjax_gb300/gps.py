"""GP prior and conjugate posterior (mirrors gpjax/gps.py:56-743)."""
from __future__ import annotations

import torch

from . import _lib
from .config import precision_code
from .distributions import GaussianDistribution
from .likelihoods import Gaussian
from .linalg import Dense, add_jitter, psd
from .mean_functions import Constant, Zero


class AbstractPrior:
    def __init__(self, kernel, mean_function=None, jitter: float = 1e-6):
        self.kernel = kernel
        self.mean_function = mean_function if mean_function is not None else Zero()
        self.jitter = jitter


class Prior(AbstractPrior):
    """GP prior p(f) (gps.py:81-254)."""

    def __mul__(self, other):
        return construct_posterior(prior=self, likelihood=other)

    __rmul__ = __mul__

    def predict(self, test_inputs: torch.Tensor) -> GaussianDistribution:
        """N(m(t), K(t, t) + jitter I) (gps.py:223-254)."""
        mean = self.mean_function(test_inputs)[:, 0]
        Ktt = self.kernel.gram(test_inputs).to_dense()
        return GaussianDistribution(mean, psd(Dense(add_jitter(Ktt, self.jitter))))


class AbstractPosterior:
    def __init__(self, prior: AbstractPrior, likelihood, jitter: float = 1e-6):
        self.prior = prior
        self.likelihood = likelihood
        self.jitter = jitter

    def __call__(self, test_inputs, train_data):
        return self.predict(test_inputs, train_data)


class ConjugatePosterior(AbstractPosterior):
    """Posterior under a Gaussian likelihood (gps.py:378-526)."""

    def predict(self, test_inputs: torch.Tensor, train_data, precision: str | None = None,
                full_covariance: bool = True) -> GaussianDistribution:
        """Predictive N(mean, cov) at test_inputs (gps.py:443-526).

        One fused call (gpk_predict) computes the mean, the predictive variance
        and, when ``full_covariance`` is true, the full t x t covariance; with
        ``full_covariance=False`` only its diagonal is formed.
        """
        kernel = self.prior.kernel
        x = kernel.slice_input(train_data.X)
        t = kernel.slice_input(test_inputs.to(train_data.X.device, torch.float64))
        y = train_data.y.reshape(-1)
        dev = _lib.require_cuda(x, t, y)
        n, m, d = x.shape[0], t.shape[0], x.shape[1]
        const = _mean_constant(self.prior.mean_function, dev)
        theta = kernel.theta_vector(dev, self.likelihood.obs_stddev.value, const).detach()
        prec = precision_code(precision)
        mean = torch.empty(m, dtype=torch.float64, device=dev)
        var = torch.empty(m, dtype=torch.float64, device=dev)
        cov = torch.empty((m, m), dtype=torch.float64, device=dev) if full_covariance else None
        info = torch.zeros(1, dtype=torch.int32, device=dev)
        xc, tc, yc = x.detach().contiguous(), t.detach().contiguous(), y.detach().contiguous()
        nbytes = _lib.lib().gpk_predict_workspace_bytes(n, m, d, prec)
        ws = _lib.workspace(nbytes, dev)
        _lib.call("gpk_predict", kernel.kind, n, m, d, xc.data_ptr(), d, yc.data_ptr(),
                  tc.data_ptr(), d, theta.data_ptr(), kernel.n_ls, float(self.jitter),
                  float(self.prior.jitter), prec, mean.data_ptr(), var.data_ptr(),
                  _lib.ptr(cov), m, info.data_ptr(), ws.data_ptr(), ws.numel(),
                  _lib.stream_ptr(dev))
        dist = GaussianDistribution(mean, psd(Dense(cov)) if cov is not None else None)
        dist._variance = var
        dist.info = info
        return dist


def _mean_constant(mean_function, device) -> torch.Tensor:
    if isinstance(mean_function, Constant):
        return mean_function.value_tensor(device)
    raise TypeError("only Constant / Zero mean functions are supported on the GPU path")


def construct_posterior(prior: Prior, likelihood) -> ConjugatePosterior:
    """prior * likelihood (gps.py:724-743)."""
    if isinstance(likelihood, Gaussian):
        return ConjugatePosterior(prior=prior, likelihood=likelihood)
    raise NotImplementedError("only the Gaussian (conjugate) likelihood is on the GPU path")
