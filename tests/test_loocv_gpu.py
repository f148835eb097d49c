"""GPU parity of conjugate_loocv (gpjax/objectives.py:110-178) and its gradient
against the float64 oracle (LU solve and inverse, torch float64 autograd)."""
import numpy as np
import pytest

import gpjax_gb300 as gpx
from oracle import gp_oracle as O
from tests._gpu_helpers import grads_of, make_posterior, to_cuda_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,n,d,ard", [(0, 1, 1, False), (0, 17, 2, True), (1, 130, 3, True),
                                          (2, 300, 8, True), (2, 700, 4, False)])
def test_loocv_parity(cuda_lib, kind, n, d, ard):
    rng = np.random.default_rng(n + d)
    x = rng.uniform(-2, 2, (n, d))
    y = (np.sin(x).sum(1) + 0.1 * rng.standard_normal(n))[:, None]
    ls = np.exp(rng.uniform(np.log(0.5), np.log(2.0), d)) if ard else np.array(1.2)
    var, sd, c = 1.1, 0.2, 0.1
    post = to_cuda_params(make_posterior(kind, ls, var, sd, c))
    val = gpx.objectives.conjugate_loocv(post, gpx.Dataset(X=x, y=y))
    val.backward()
    g = grads_of(post)
    ref, gr = O.conjugate_loocv_torch(kind, x, y, ls, var, sd, c)
    gref = np.concatenate([np.atleast_1d(gr["lengthscale"]),
                           [gr["variance"], gr["obs_stddev"], gr["constant"]]])
    assert abs(float(val.detach()) - ref) <= 1e-10 * max(1.0, abs(ref)), (float(val), ref)
    assert np.allclose(g, gref, rtol=1e-7, atol=1e-8 * max(1.0, np.abs(gref).max())), (g, gref)
