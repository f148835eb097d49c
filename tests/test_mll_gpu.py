"""GPU parity of conjugate_mll and its gradient against the float64 oracle
(LU-based value as in the reference, torch float64 autograd gradients).

Tolerances: plain FP64 form 1e-10 relative on the MLL, 1e-7 on gradients;
mixed form 1e-6 relative on the MLL and 1e-4 relative (to the gradient norm
and per component with a small absolute floor) on gradients."""
import numpy as np
import pytest
import torch

import gpjax_gb300 as gpx
from oracle import gp_oracle as O
from tests._gpu_helpers import c2_like, grads_of, make_posterior, to_cuda_params

pytestmark = pytest.mark.gpu


def run(kind, x, y, ls, var, sd, c, precision):
    post = to_cuda_params(make_posterior(kind, ls, var, sd, c))
    data = gpx.Dataset(X=x, y=y)
    val = gpx.objectives.conjugate_mll(post, data, precision=precision)
    val.backward()
    return float(val), grads_of(post)


def oracle(kind, x, y, ls, var, sd, c):
    val = O.conjugate_mll(kind, x, y, ls, var, sd, c)
    _, g = O.conjugate_mll_torch(kind, x, y, ls, var, sd, c, lu=False)
    return val, np.concatenate([np.atleast_1d(g["lengthscale"]),
                                [g["variance"], g["obs_stddev"], g["constant"]]])


CASES = [(0, 1, 1), (1, 2, 2), (2, 3, 1), (0, 17, 3), (2, 63, 8), (1, 65, 4), (2, 127, 8),
         (0, 129, 2), (2, 300, 8), (1, 555, 5), (2, 1000, 8), (0, 1100, 16)]


@pytest.mark.parametrize("kind,n,d", CASES)
@pytest.mark.parametrize("ard", [True, False])
def test_mll_fp64_parity(cuda_lib, kind, n, d, ard):
    rng = np.random.default_rng(n * 7 + d)
    x = rng.uniform(-2, 2, size=(n, d))
    y = np.sin(x).sum(1, keepdims=True) + 0.1 * rng.standard_normal((n, 1))
    ls = np.exp(rng.uniform(np.log(0.5), np.log(2.0), d)) if ard else np.array(1.3)
    var, sd, c = 1.2, 0.3, 0.1
    val, g = run(kind, x, y, ls, var, sd, c, "fp64")
    ref, gref = oracle(kind, x, y, ls, var, sd, c)
    assert abs(val - ref) <= 1e-10 * max(1.0, abs(ref)), (val, ref)
    assert np.allclose(g, gref, rtol=1e-7, atol=1e-8 * max(1.0, np.abs(gref).max())), (g, gref)


def _mixed_check(val, g, ref, gref, tol_scale, gtol=1e-4, vtol=1e-6, ptol=1e-3):
    """MLL within 1e-6 of tol_scale; gradient within gtol relative to its norm
    (the mixed form's factor carries float32 backward error, which bounds the
    trace term of the noise gradient; each component is also held to ptol)."""
    err = np.abs(g - gref)
    assert abs(val - ref) <= vtol * tol_scale, (val, ref, abs(val - ref) / tol_scale)
    assert np.linalg.norm(err) <= gtol * np.linalg.norm(gref), (g, gref)
    assert np.all(err <= ptol * np.abs(gref) + gtol * 0.1 * np.linalg.norm(gref)), (g, gref)


# n = 4500 puts 2304-wide nodes at the top of the recursion (128 x 256 GEMM tiles)
@pytest.mark.parametrize("n", [700, 2048, 3000, 4500])
def test_mll_mixed_parity_c2(cuda_lib, n):
    """Matern-5/2 ARD, d = 8, X ~ N(0, I), noise 1e-2: |dMLL|/|MLL| <= 1e-6."""
    x, y, ls = c2_like(n, 8, seed=n, kind=2)
    val, g = run(2, x, y, ls, 1.0, 0.1, 0.0, "mixed")
    ref, gref = oracle(2, x, y, ls, 1.0, 0.1, 0.0)
    _mixed_check(val, g, ref, gref, abs(ref))


@pytest.mark.parametrize("kind,n,d", [(1, 1500, 6), (0, 555, 16), (1, 2600, 5)])
def test_mll_mixed_parity_other_kernels(cuda_lib, kind, n, d):
    """RBF and Matern-3/2 at the mixed form's targets: |dMLL|/|MLL| <= 1e-6 and
    the gradient within 1e-4 of its norm (condition numbers up to ~4e3)."""
    x, y, ls = c2_like(n, d, seed=n, kind=kind)
    val, g = run(kind, x, y, ls, 1.0, 0.1, 0.0, "mixed")
    ref, gref = oracle(kind, x, y, ls, 1.0, 0.1, 0.0)
    _mixed_check(val, g, ref, gref, abs(ref))


def test_mll_mixed_near_cancelling_mll(cuda_lib):
    """RBF, d = 4, n = 1024, condition number ~1e4, where the MLL (8.4) is the
    difference of terms three orders of magnitude larger (log det ~ -4e3,
    quadratic ~1e3, n log 2 pi / 2 ~ 940): the MLL is held to 1e-6 of the size
    of its terms; the gradient, whose noise component is the difference of
    alpha^T alpha (5e4) and tr(Sigma^-1), to 3e-4 of its norm -- the float32
    rounding of the Gram entries that the refinement's residual reads moves
    alpha by ~1e-4 relative at this conditioning."""
    x, y, ls = c2_like(1024, 4, seed=1024, kind=0)
    val, g = run(0, x, y, ls, 1.0, 0.1, 0.0, "mixed")
    ref, gref = oracle(0, x, y, ls, 1.0, 0.1, 0.0)
    S = O.gram(0, x, ls, 1.0) + (1e-6 + 1e-2) * np.eye(1024)
    ld = np.linalg.slogdet(S)[1]
    quad = float(y[:, 0] @ np.linalg.solve(S, y[:, 0]))
    _mixed_check(val, g, ref, gref, 0.5 * (abs(ld) + abs(quad) + 1024 * np.log(2 * np.pi)),
                 gtol=3e-4, vtol=1e-6, ptol=5e-3)


def test_mll_matches_finite_differences(cuda_lib):
    x, y, ls = c2_like(200, 3, seed=5)
    var, sd, c = 0.9, 0.2, 0.05
    _, g = run(2, x, y, ls, var, sd, c, "fp64")
    vec = np.concatenate([ls, [var, sd, c]])

    def f(v):
        post = make_posterior(2, v[:3], v[3], v[4], v[5])
        return float(gpx.objectives.conjugate_mll(post, gpx.Dataset(X=x, y=y), precision="fp64"))
    fd = O.central_fd(f, vec, 1e-6)
    assert np.allclose(g, fd, rtol=1e-5, atol=1e-5), (g, fd)


def test_mll_not_pd_gives_nan_and_info(cuda_lib):
    # duplicate inputs with zero noise and zero jitter: singular Sigma
    x = np.zeros((5, 2))
    y = np.ones((5, 1))
    post = make_posterior(0, [1.0, 1.0], 1.0, 0.0, 0.0, jitter=0.0)
    val = gpx.objectives.conjugate_mll(post, gpx.Dataset(X=x, y=y), precision="fp64")
    assert np.isnan(float(val))


def test_mll_deterministic(cuda_lib):
    x, y, ls = c2_like(600, 8, seed=11)
    a, ga = run(2, x, y, ls, 1.0, 0.1, 0.0, "mixed")
    b, gb = run(2, x, y, ls, 1.0, 0.1, 0.0, "mixed")
    assert a == b and np.array_equal(ga, gb)


@pytest.mark.parametrize("n", [4500])
def test_mll_mixed_dirty_workspace(cuda_lib, n):
    """The mixed form must not depend on the workspace's prior contents: run it
    through the C ABI on a workspace filled with a finite non-zero byte pattern
    (float32 785.07), at a size whose recursion has 2304-wide nodes (256-wide
    GEMM tiles over triangular operands), and compare with a clean workspace
    and the oracle."""
    from gpjax_gb300 import _lib
    x, y, ls = c2_like(n, 8, seed=n + 1, kind=2)
    dev = torch.device("cuda", 0)
    theta = torch.tensor(list(ls) + [1.0, 0.1, 0.0], dtype=torch.float64, device=dev)
    X = torch.as_tensor(x, device=dev)
    Y = torch.as_tensor(y[:, 0], device=dev).contiguous()
    nbytes = _lib.lib().gpk_conjugate_mll_workspace_bytes(n, 8, _lib.PREC_MIXED)
    results = []
    for fill in (0x00, 0x44):
        ws = torch.full((nbytes,), fill, dtype=torch.uint8, device=dev)
        out = torch.zeros(1, dtype=torch.float64, device=dev)
        grad = torch.zeros(11, dtype=torch.float64, device=dev)
        info = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.call("gpk_conjugate_mll", _lib.MATERN52, n, 8, X.data_ptr(), 8, Y.data_ptr(),
                  theta.data_ptr(), 8, 1e-6, _lib.PREC_MIXED, 1, out.data_ptr(),
                  grad.data_ptr(), info.data_ptr(), ws.data_ptr(), ws.numel(),
                  _lib.stream_ptr(dev))
        torch.cuda.synchronize(dev)
        assert int(info.item()) == 0
        results.append((float(out.item()), grad.cpu().numpy().copy()))
    ref = O.conjugate_mll(2, x, y, ls, 1.0, 0.1, 0.0)
    (v0, g0), (v1, g1) = results
    assert abs(v1 - ref) <= 1e-6 * abs(ref), (v1, ref)
    assert v1 == v0 and np.array_equal(g1, g0)


@pytest.mark.parametrize("kind", [O.MATERN12, O.rational_quadratic(0.8)])
@pytest.mark.parametrize("n,d", [(400, 3), (1100, 5)])
def test_mll_added_kernels(cuda_lib, kind, n, d):
    """Matern12 and RationalQuadratic: float64 form at the float64 tolerances;
    mixed form at 1e-6 relative on the MLL and 1e-4 on the gradient norm
    (|MLL| between 110 and 1400 on these draws)."""
    from gpjax_gb300 import kernels as K
    rng = np.random.default_rng(n + d)
    x = rng.standard_normal((n, d))
    ls = np.exp(rng.uniform(np.log(0.5), np.log(3.0), d))
    S = O.gram(kind, x, ls, 1.0) + (1e-6 + 1e-2) * np.eye(n)
    y = (np.linalg.cholesky(S) @ rng.standard_normal(n))[:, None]
    ref, gref = oracle(kind, x, y, ls, 1.0, 0.1, 0.05)
    for prec, vtol, gtol in (("fp64", 1e-10, 1e-7), ("mixed", 1e-6, 1e-4)):
        if isinstance(kind, tuple):
            kern = K.RationalQuadratic(lengthscale=ls, variance=1.0, alpha=kind[1])
        else:
            kern = K.Matern12(lengthscale=ls, variance=1.0)
        prior = gpx.gps.Prior(kernel=kern, mean_function=gpx.mean_functions.Constant(
            gpx.parameters.Real(0.05)), jitter=1e-6)
        post = to_cuda_params(prior * gpx.likelihoods.Gaussian(num_datapoints=n, obs_stddev=0.1))
        val = gpx.objectives.conjugate_mll(post, gpx.Dataset(X=x, y=y), precision=prec)
        val.backward()
        g = grads_of(post)
        assert abs(float(val.detach()) - ref) <= vtol * abs(ref), (prec, float(val), ref)
        assert np.linalg.norm(g - gref) <= gtol * np.linalg.norm(gref), (prec, g, gref)


@pytest.mark.parametrize("precision,vtol,gtol", [("fp64", 1e-10, 1e-7), ("mixed", 1e-6, 1e-4)])
def test_mll_c2_generator_n8192(cuda_lib, precision, vtol, gtol):
    """The benchmark's generator (Matern-5/2 ARD, d = 8, X ~ N(0, I), log-uniform
    lengthscales in [0.3, 3], noise 1e-2, y a float64 prior sample) at n = 8192,
    both forms against the float64 oracle (the reference's LU op sequence)."""
    import bench
    n, d = 8192, 8
    x, ls, eps = bench.c2_inputs(n, d, 1)
    y = bench.c2_y_host(x, ls, eps)[:, None]
    ref, g = O.conjugate_mll_grad_lu(O.MATERN52, x, y, ls, 1.0, 0.1, 0.0)
    gref = np.concatenate([g["lengthscale"], [g["variance"], g["obs_stddev"], g["constant"]]])
    val, gg = run(2, x, y, ls, 1.0, 0.1, 0.0, precision)
    assert abs(val - ref) <= vtol * abs(ref), (precision, val, ref, abs(val - ref) / abs(ref))
    assert np.linalg.norm(gg - gref) <= gtol * np.linalg.norm(gref), (precision, gg, gref)
