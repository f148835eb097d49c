"""GPU: the reference's CPU configuration exactly -- n = 2048 training points,
X ~ U[-3, 3]^4, y = sum_j sin(2 x_j) + N(0, 0.1^2), 512 test points from the
same distribution, RBF with lengthscale 1, variance 1, noise variance 0.01
(obs_stddev 0.1) -- in both forms: conjugate_mll and its gradient, and the
predictive mean and variance, against the float64 oracle.

Tolerances: float64 form 1e-10 relative on the MLL and 1e-7 on the gradient;
mixed form 1e-6 relative on the MLL and 1e-4 relative to the gradient's norm
(the mixed form's targets); predictive mean / variance 1e-9 (float64) and
1e-4 of their scale (mixed)."""
import numpy as np
import pytest
import torch

import gpjax_gb300 as gpx
from oracle import gp_oracle as O
from tests._gpu_helpers import grads_of, make_posterior, to_cuda_params

pytestmark = pytest.mark.gpu


def c1_data(seed=0):
    rng = np.random.default_rng(seed)
    n, d = 2048, 4
    x = rng.uniform(-3, 3, (n, d))
    y = (np.sin(2 * x).sum(1) + 0.1 * rng.standard_normal(n))[:, None]
    xt = rng.uniform(-3, 3, (512, d))
    return x, y, xt


@pytest.fixture(scope="module")
def c1_reference():
    x, y, xt = c1_data()
    val, g = O.conjugate_mll_torch(O.RBF, x, y, np.array(1.0), 1.0, 0.1, 0.0, lu=True)
    gref = np.array([g["lengthscale"], g["variance"], g["obs_stddev"], g["constant"]], float)
    mean, cov = O.predict(O.RBF, x, y, xt, 1.0, 1.0, 0.1, 0.0)
    return x, y, xt, val, gref, mean, np.diag(cov)


@pytest.mark.parametrize("precision,vtol,gtol", [("fp64", 1e-10, 1e-7), ("mixed", 1e-6, 1e-4)])
def test_c1_mll_and_gradient(cuda_lib, c1_reference, precision, vtol, gtol):
    x, y, _, ref, gref, _, _ = c1_reference
    post = to_cuda_params(make_posterior(O.RBF, np.array(1.0), 1.0, 0.1, 0.0))
    val = gpx.objectives.conjugate_mll(post, gpx.Dataset(X=x, y=y), precision=precision)
    val.backward()
    g = grads_of(post)
    rel = abs(float(val.detach()) - ref) / abs(ref)
    assert rel <= vtol, (precision, float(val), ref, rel)
    assert np.linalg.norm(g - gref) <= gtol * np.linalg.norm(gref), (precision, g, gref)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-4)])
def test_c1_predict(cuda_lib, c1_reference, precision, tol):
    x, y, xt, _, _, mean, var = c1_reference
    post = make_posterior(O.RBF, np.array(1.0), 1.0, 0.1, 0.0)
    dist = post.predict(torch.as_tensor(xt, device="cuda"), gpx.Dataset(X=x, y=y),
                        precision=precision, full_covariance=False)
    m, v = dist.mean.cpu().numpy(), dist.variance.cpu().numpy()
    assert np.allclose(m, mean, rtol=tol, atol=tol * np.abs(mean).max())
    assert np.allclose(v, var, rtol=tol, atol=tol * np.abs(var).max())
