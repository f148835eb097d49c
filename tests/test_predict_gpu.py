"""GPU parity of ConjugatePosterior.predict (mean, variance, covariance)."""
import numpy as np
import pytest
import torch

import gpjax_gb300 as gpx
from oracle import gp_oracle as O
from tests._gpu_helpers import c2_like, make_posterior

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,n,t,d", [(0, 1, 1, 1), (2, 50, 7, 3), (1, 300, 64, 4),
                                        (0, 2048, 512, 4)])
def test_predict_fp64(cuda_lib, kind, n, t, d):
    rng = np.random.default_rng(n + t)
    x = rng.uniform(-3, 3, size=(n, d))
    y = np.sin(2 * x).sum(1, keepdims=True) + 0.1 * rng.standard_normal((n, 1))
    xt = rng.uniform(-3, 3, size=(t, d))
    post = make_posterior(kind, 1.0, 1.0, 0.1, 0.2)
    dist = post.predict(torch.as_tensor(xt, device="cuda"), gpx.Dataset(X=x, y=y),
                        precision="fp64")
    mean, cov = O.predict(kind, x, y, xt, 1.0, 1.0, 0.1, 0.2)
    assert np.allclose(dist.mean.cpu().numpy(), mean, rtol=1e-9, atol=1e-9)
    assert np.allclose(dist.variance.cpu().numpy(), np.diag(cov), rtol=1e-8, atol=1e-9)
    assert np.allclose(dist.covariance().cpu().numpy(), cov, rtol=1e-8, atol=1e-9)


def test_predict_mixed(cuda_lib):
    x, y, ls = c2_like(1500, 8, seed=3)
    xt = np.random.default_rng(4).standard_normal((200, 8))
    post = make_posterior(2, ls, 1.0, 0.1, 0.0)
    dist = post.predict(torch.as_tensor(xt, device="cuda"), gpx.Dataset(X=x, y=y),
                        precision="mixed", full_covariance=False)
    mean, cov = O.predict(2, x, y, xt, ls, 1.0, 0.1, 0.0)
    assert np.allclose(dist.mean.cpu().numpy(), mean, rtol=1e-4, atol=1e-4 * np.abs(mean).max())
    assert np.allclose(dist.variance.cpu().numpy(), np.diag(cov), atol=1e-4)


@pytest.mark.parametrize("kind,n,t,d,tol", [(2, 1500, 300, 8, 1e-6), (0, 4500, 257, 4, 1e-5),
                                            (1, 700, 1, 3, 1e-6)])
def test_predict_mean_variance_tensor_core_path(cuda_lib, kind, n, t, d, tol):
    """Mean and variance without the covariance run on the mixed form's
    tensor-core factorisation (Q^T = Ktx M^T as one split-TF32 GEMM whose
    epilogue keeps only the row sums of squares); n = 4500 includes the
    split-float16 wide nodes.  The RBF d = 4 case is the ill-conditioned one
    (measured 6.4e-6 on the mean, 4.4e-6 on the variance; the Matern-5/2
    d = 8 case 1.4e-7 / 1.1e-7)."""
    rng = np.random.default_rng(n + t + kind)
    x = rng.uniform(-2, 2, size=(n, d))
    y = np.sin(2 * x).sum(1, keepdims=True) + 0.1 * rng.standard_normal((n, 1))
    xt = rng.uniform(-2.2, 2.2, size=(t, d))
    ls = np.exp(rng.uniform(np.log(0.5), np.log(1.5), d))
    post = make_posterior(kind, ls, 1.3, 0.1, 0.2)
    dist = post.predict(torch.as_tensor(xt, device="cuda"), gpx.Dataset(X=x, y=y),
                        precision="mixed", full_covariance=False)
    mean, cov = O.predict(kind, x, y, xt, ls, 1.3, 0.1, 0.2)
    m = dist.mean.cpu().numpy()
    v = dist.variance.cpu().numpy()
    merr = np.max(np.abs(m - mean)) / np.max(np.abs(mean))
    verr = np.max(np.abs(v - np.diag(cov)))
    print("mean rel", merr, "var abs", verr)
    assert merr <= tol and verr <= tol, (merr, verr)
