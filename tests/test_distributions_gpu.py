"""GPU: GaussianDistribution with a Dense covariance (distributions.py:42-134)
against scipy's multivariate normal -- the reference's check of its Dense
log_prob, entropy, variance and covariance against numpyro's
MultivariateNormal (tests/test_gaussian_distribution.py:102-123), restated:
n in {1, 2, 5, 100}, mean ~ U[0, 1]^n, covariance S S^T with S ~ U[0, 1]^{n x n},
y ~ U[0, 1]^n.  The reference's bound is an absolute 1e-5 on the norm of the
difference; here it is 1e-8 relative."""
import numpy as np
import pytest
import torch
from scipy import stats

from gpjax_gb300.distributions import GaussianDistribution
from gpjax_gb300.linalg import Dense

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 5, 100])
def test_dense_gaussian_matches_mvn(cuda_lib, n):
    rng = np.random.default_rng(42 + n)
    mean = rng.uniform(size=n)
    sqrt = rng.uniform(size=(n, n))
    cov = sqrt @ sqrt.T
    y = rng.uniform(size=n)
    dev = torch.device("cuda")
    dist = GaussianDistribution(torch.as_tensor(mean, device=dev),
                                Dense(torch.as_tensor(cov, device=dev)))
    ref = stats.multivariate_normal(mean=mean, cov=cov)
    lp = float(dist.log_prob(torch.as_tensor(y, device=dev)))
    assert abs(lp - ref.logpdf(y)) <= 1e-7 * max(1.0, abs(ref.logpdf(y)))
    assert abs(float(dist.entropy()) - ref.entropy()) <= 1e-8 * max(1.0, abs(ref.entropy()))
    assert np.allclose(dist.mean.cpu().numpy(), mean)
    assert np.allclose(dist.variance.cpu().numpy(), np.diag(cov), rtol=1e-12)
    assert np.allclose(dist.covariance().cpu().numpy(), cov, rtol=1e-12)
