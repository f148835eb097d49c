"""GPU: the training loops (gpjax/fit.py:183-361) over the library's
conjugate_mll land where the same optimiser lands on the float64 oracle's
objective, from the same start, in the reference's unconstrained coordinates
(softplus for lengthscale, variance and obs_stddev; identity for the mean)."""
import numpy as np
import pytest
import torch
from scipy.optimize import minimize

import gpjax_gb300 as gpx
from oracle import gp_oracle as O
from tests._gpu_helpers import make_posterior

pytestmark = pytest.mark.gpu


def _sp(u):
    return np.log1p(np.exp(u))


def _sp_inv(v):
    return v + np.log(-np.expm1(-v))


def _oracle_loss(u, kind, x, y, d):
    ls, var, sd, c = _sp(u[:d]), _sp(u[d]), _sp(u[d + 1]), u[d + 2]
    val, g = O.conjugate_mll_torch(kind, x, y, ls, var, sd, c, lu=False)
    sig = 1.0 / (1.0 + np.exp(-u[: d + 2]))
    grad = np.concatenate([np.asarray(g["lengthscale"]) * sig[:d],
                           [g["variance"] * sig[d], g["obs_stddev"] * sig[d + 1], g["constant"]]])
    return -val, -grad


@pytest.mark.parametrize("runner", ["scipy", "lbfgs"])
def test_fit_matches_oracle_fit(cuda_lib, runner):
    rng = np.random.default_rng(4)
    n, d, kind = 150, 2, O.MATERN52
    x = rng.uniform(-2, 2, (n, d))
    y = (np.sin(2 * x).sum(1) + 0.1 * rng.standard_normal(n))[:, None]
    ls0, var0, sd0, c0 = np.array([1.0, 0.7]), 0.8, 0.3, 0.0
    post = make_posterior(kind, ls0, var0, sd0, c0)
    data = gpx.Dataset(X=x, y=y)
    objective = lambda p, dd: -gpx.objectives.conjugate_mll(p, dd, precision="fp64")  # noqa: E731
    u0 = np.concatenate([_sp_inv(ls0), [_sp_inv(var0), _sp_inv(sd0), c0]])
    if runner == "scipy":
        post, hist = gpx.fit.fit_scipy(model=post, objective=objective, train_data=data,
                                       max_iters=200, verbose=False)
        ref = minimize(_oracle_loss, u0, args=(kind, x, y, d), jac=True,
                       options={"maxiter": 200})
        final = hist[-1]
        assert hist[0] > final
    else:
        post, final = gpx.fit.fit_lbfgs(model=post, objective=objective, train_data=data,
                                        max_iters=200)
        ref = minimize(_oracle_loss, u0, args=(kind, x, y, d), jac=True, method="L-BFGS-B",
                       options={"maxiter": 200, "maxls": 32, "gtol": 1e-5})
    got = np.concatenate([post.prior.kernel.lengthscale.value.cpu().numpy(),
                          [float(post.prior.kernel.variance.value),
                           float(post.likelihood.obs_stddev.value),
                           float(post.prior.mean_function.constant.value)]])
    want = np.concatenate([_sp(ref.x[:d]), [_sp(ref.x[d]), _sp(ref.x[d + 1]), ref.x[d + 2]]])
    assert abs(final - ref.fun) <= 1e-6 * abs(ref.fun), (final, ref.fun)
    assert np.allclose(got, want, rtol=1e-3, atol=1e-4), (got, want)
    # the optimum: the library's gradient there is ~0 in every coordinate
    for p in (post.prior.kernel.lengthscale, post.prior.kernel.variance,
              post.likelihood.obs_stddev):
        p.to("cuda").requires_grad_(True)
    val = gpx.objectives.conjugate_mll(post, data, precision="fp64")
    val.backward()
    assert float(post.likelihood.obs_stddev.value.grad.abs()) < 1e-2 * n
    assert torch.isfinite(val)
