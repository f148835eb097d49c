"""Shared helpers of the GPU parity tests."""
import numpy as np
import torch

import gpjax_gb300 as gpx
from gpjax_gb300 import kernels as K

KINDS = {0: K.RBF, 1: K.Matern32, 2: K.Matern52}


def make_posterior(kind, ls, var, sd, c, jitter=1e-6):
    kern = KINDS[kind](lengthscale=np.asarray(ls, np.float64), variance=var)
    prior = gpx.gps.Prior(kernel=kern, mean_function=gpx.mean_functions.Constant(
        gpx.parameters.Real(c)), jitter=jitter)
    lik = gpx.likelihoods.Gaussian(num_datapoints=1, obs_stddev=sd)
    return prior * lik


def c2_like(n, d, seed, kind=2):
    """C2-style data: X ~ N(0, I), log-uniform ARD lengthscales in [0.3, 3],
    y drawn from the prior plus noise (float64)."""
    from oracle import gp_oracle as O
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, d))
    ls = np.exp(rng.uniform(np.log(0.3), np.log(3.0), d))
    S = O.gram(kind, x, ls, 1.0) + (1e-6 + 1e-2) * np.eye(n)
    y = np.linalg.cholesky(S) @ rng.standard_normal(n)
    return x, y[:, None], ls


def grads_of(post):
    g_ls = post.prior.kernel.lengthscale.value.grad
    return np.concatenate([np.atleast_1d(g_ls.cpu().numpy()),
                           [float(post.prior.kernel.variance.value.grad),
                            float(post.likelihood.obs_stddev.value.grad),
                            float(post.prior.mean_function.constant.value.grad)]])


def to_cuda_params(post):
    for p in (post.prior.kernel.lengthscale, post.prior.kernel.variance,
              post.likelihood.obs_stddev, post.prior.mean_function.constant):
        p.to("cuda").requires_grad_(True)
    return post
