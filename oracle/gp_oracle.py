"""Float64 CPU oracle for the exact- and sparse-GP hot path of GPJax 0.13.2.

TEST INFRASTRUCTURE ONLY.  This module is the checker that the CUDA path is
compared against.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it; the
product package ``gpjax_gb300`` never does.

It restates, in numpy/scipy float64, the op sequence of the reference:

* kernels      -- ``gpjax/kernels/stationary/rbf.py:40-44``,
                  ``matern32.py:41-54``, ``matern52.py:42-53``,
                  ``utils.py:42-67`` (``squared_distance`` and the 1e-36 floor
                  of ``euclidean_distance``)
* Gram / cross -- ``gpjax/kernels/computations/dense.py:32-36``,
                  ``base.py:56-109``
* jitter       -- ``gpjax/linalg/utils.py:39-65``
* log_prob     -- ``gpjax/distributions.py:115-134`` with the Dense branches
                  of ``logdet`` (``slogdet``, an LU) and ``solve``
                  (``jnp.linalg.solve``, a second LU) at
                  ``gpjax/linalg/operations.py:109-111,163-165``
* conjugate_mll   -- ``gpjax/objectives.py:93-107``
* collapsed_elbo  -- ``gpjax/objectives.py:341-416``
* predict         -- ``gpjax/gps.py:494-526``
* SGPR predict    -- ``gpjax/variational_families.py:786-870``

Gradients stand in for ``jax.grad`` of the reference: the same op sequence is
re-run under torch float64 autograd (``*_torch`` functions), with the
parameters in the reference's constrained coordinates (``lengthscale``,
``variance``, ``obs_stddev``, the constant mean, the inducing inputs).
Central finite differences (``central_fd``) cross-check both.

Parity status: GPJax pins no golden value for these functions (its tests check
shapes and identities only), and JAX cannot run where this oracle is built, so
the oracle is pinned by the reference's own known-answer cases and identities:
the 2x2 solve/logdet/Cholesky cases of ``tests/test_linalg.py:237-396``,
``log_prob`` == the multivariate-normal log-density
(``tests/test_gaussian_distribution.py:102-123``) and
``collapsed_elbo(Z = X) == conjugate_mll`` (``tests/test_objectives.py:193-199``).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla

RBF, MATERN32, MATERN52, MATERN12, RATIONAL_QUADRATIC = 0, 1, 2, 3, 4
KERNEL_NAMES = {RBF: "RBF", MATERN32: "Matern32", MATERN52: "Matern52", MATERN12: "Matern12",
                RATIONAL_QUADRATIC: "RationalQuadratic"}


def rational_quadratic(alpha: float):
    """Kernel code of a rational quadratic with shape alpha (the other kernels
    are plain integer codes)."""
    return (RATIONAL_QUADRATIC, float(alpha))


def _kind(kind):
    """(integer kernel code, rational-quadratic alpha or None)."""
    if isinstance(kind, tuple):
        return int(kind[0]), float(kind[1])
    return int(kind), None
DEFAULT_JITTER = 1e-6  # gpjax/gps.py:68,344 and variational_families.py:118
_FLOOR = 1e-36  # gpjax/kernels/stationary/utils.py:67


# --------------------------------------------------------------------------
# Kernels (numpy float64)
# --------------------------------------------------------------------------
def _sqdist(x: np.ndarray, y: np.ndarray, ls) -> np.ndarray:
    """sum_j (x_j/l_j - y_j/l_j)^2 for all pairs (rbf.py:41-43, utils.py:53)."""
    ls = np.broadcast_to(np.asarray(ls, np.float64), (x.shape[1],))
    xs = x / ls
    ys = y / ls
    out = np.zeros((x.shape[0], y.shape[0]))
    for j in range(x.shape[1]):
        out += (xs[:, None, j] - ys[None, :, j]) ** 2
    return out


def kernel_from_sqdist(kind: int, sq: np.ndarray, variance: float) -> np.ndarray:
    """Pointwise kernel value from the scaled squared distance."""
    kind, alpha = _kind(kind)
    if kind == RBF:  # rbf.py:43
        return variance * np.exp(-0.5 * sq)
    if kind == RATIONAL_QUADRATIC:  # rational_quadratic.py:76-83
        return variance * (1.0 + 0.5 * sq / alpha) ** (-alpha)
    tau = np.sqrt(np.maximum(sq, _FLOOR))  # utils.py:67
    if kind == MATERN12:  # matern12.py:44-48
        return variance * np.exp(-tau)
    if kind == MATERN32:  # matern32.py:48-53
        return variance * (1.0 + np.sqrt(3.0) * tau) * np.exp(-np.sqrt(3.0) * tau)
    if kind == MATERN52:  # matern52.py:46-52
        return (variance * (1.0 + np.sqrt(5.0) * tau + 5.0 / 3.0 * tau**2)
                * np.exp(-np.sqrt(5.0) * tau))
    raise ValueError(f"unknown kernel kind {kind}")


def cross_covariance(kind, x, y, ls, variance) -> np.ndarray:
    """K[i, j] = k(x_i, y_j) (computations/dense.py:32-36)."""
    x = np.atleast_2d(np.asarray(x, np.float64))
    y = np.atleast_2d(np.asarray(y, np.float64))
    return kernel_from_sqdist(kind, _sqdist(x, y, ls), variance)


def gram(kind, x, ls, variance) -> np.ndarray:
    """Full-square Gram (computations/base.py:56-72)."""
    return cross_covariance(kind, x, x, ls, variance)


def diagonal(kind, x, ls, variance) -> np.ndarray:
    """diag k(x_i, x_i) (computations/base.py:95-109)."""
    return np.array([kernel_from_sqdist(kind, np.zeros((1, 1)), variance)[0, 0]] * len(x))


def add_jitter(K: np.ndarray, jitter: float) -> np.ndarray:
    """K + I*jitter (linalg/utils.py:39-65)."""
    return K + np.eye(K.shape[0]) * jitter


# --------------------------------------------------------------------------
# Distributions / linear algebra (the reference's Dense branches)
# --------------------------------------------------------------------------
def logdet_dense(A: np.ndarray) -> float:
    """slogdet(A)[1] via LU (linalg/operations.py:163-165)."""
    return float(np.linalg.slogdet(A)[1])


def solve_dense(A: np.ndarray, b: np.ndarray) -> np.ndarray:
    """jnp.linalg.solve (LU) with the vector reshape of operations.py:90-94,117-118."""
    return np.linalg.solve(A, b)


def gaussian_log_prob(mu: np.ndarray, Sigma: np.ndarray, y: np.ndarray) -> float:
    """-1/2 (n log 2pi + logdet Sigma + diff^T Sigma^-1 diff) (distributions.py:124-134)."""
    n = mu.shape[-1]
    diff = y - mu
    return -0.5 * (n * np.log(2.0 * np.pi) + logdet_dense(Sigma) + diff @ solve_dense(Sigma, diff))


def conjugate_mll(kind, X, y, ls, variance, obs_stddev, mean_const=0.0,
                  jitter=DEFAULT_JITTER) -> float:
    """Exact-GP marginal log-likelihood (objectives.py:93-107).

    Sigma = (Kxx + I*jitter) + I*obs_stddev^2 -- jitter added before the noise,
    the jitter being ``posterior.prior.jitter``.
    """
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64).reshape(-1)
    obs_noise = obs_stddev**2
    mx = np.ones(X.shape[0]) * mean_const
    Kxx = gram(kind, X, ls, variance)
    Sigma = add_jitter(Kxx, jitter) + np.eye(X.shape[0]) * obs_noise
    return float(gaussian_log_prob(np.atleast_1d(mx), Sigma, np.atleast_1d(y)))


def conjugate_mll_cholesky(kind, X, y, ls, variance, obs_stddev, mean_const=0.0,
                           jitter=DEFAULT_JITTER) -> float:
    """Same quantity through a Cholesky factor (mathematically identical for SPD Sigma)."""
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64).reshape(-1)
    n = X.shape[0]
    Sigma = add_jitter(gram(kind, X, ls, variance), jitter) + np.eye(n) * obs_stddev**2
    L = np.linalg.cholesky(Sigma)
    diff = y - mean_const
    z = sla.solve_triangular(L, diff, lower=True)
    return float(-0.5 * (n * np.log(2 * np.pi) + 2.0 * np.log(np.diag(L)).sum() + z @ z))


def conjugate_loocv(kind, X, y, ls, variance, obs_stddev, mean_const=0.0,
                    jitter=DEFAULT_JITTER) -> float:
    """Leave-one-out log predictive probability (objectives.py:157-178): the
    solve and inverse of Sigma = Kxx + I (obs_var + jitter) by LU, then the sum
    of the per-point Normal log-densities."""
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64).reshape(-1, 1)
    n = X.shape[0]
    mx = np.ones((n, 1)) * mean_const  # :161
    Sigma = gram(kind, X, ls, variance) + np.eye(n) * (obs_stddev**2 + jitter)  # :164-167
    Sigma_inv_y = np.linalg.solve(Sigma, y - mx)  # :170
    Sigma_inv_diag = np.diag(np.linalg.inv(Sigma))[:, None]  # :171-172
    means = mx + (y - mx) - Sigma_inv_y / Sigma_inv_diag  # :174
    stds = np.sqrt(1.0 / Sigma_inv_diag)  # :175
    lp = -0.5 * np.log(2 * np.pi) - np.log(stds) - 0.5 * ((y - means) / stds) ** 2  # :177-178
    return float(lp.sum())


def conjugate_loocv_torch(kind, X, y, ls, variance, obs_stddev, mean_const=0.0,
                          jitter=DEFAULT_JITTER):
    """conjugate_loocv and its gradient w.r.t. (lengthscale, variance,
    obs_stddev, constant) by torch float64 autograd of the same sequence."""
    torch = _torch()
    Xt = torch.as_tensor(np.asarray(X, np.float64))
    yt = torch.as_tensor(np.asarray(y, np.float64).reshape(-1, 1))
    n = Xt.shape[0]
    ls_t, var_t, sd_t, c_t = _params(ls, variance, obs_stddev, mean_const, Xt.shape[1])
    Sigma = _t_kernel(kind, Xt, Xt, ls_t, var_t) + torch.eye(n, dtype=torch.float64) * (
        sd_t**2 + jitter)
    diff = yt - c_t
    siy = torch.linalg.solve(Sigma, diff)
    sid = torch.diagonal(torch.linalg.inv(Sigma))[:, None]
    means = c_t + diff - siy / sid
    stds = torch.sqrt(1.0 / sid)
    lp = -0.5 * math.log(2 * math.pi) - torch.log(stds) - 0.5 * ((yt - means) / stds) ** 2
    val = lp.sum()
    val.backward()
    grads = {"lengthscale": ls_t.grad.numpy().copy(), "variance": float(var_t.grad),
             "obs_stddev": float(sd_t.grad), "constant": float(c_t.grad)}
    return float(val.detach()), grads


def collapsed_elbo(kind, X, y, Z, ls, variance, obs_stddev, mean_const=0.0,
                   jitter=DEFAULT_JITTER) -> float:
    """Titsias collapsed bound, same op order as objectives.py:341-416."""
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64).reshape(-1, 1)
    Z = np.asarray(Z, np.float64)
    n = X.shape[0]
    m = Z.shape[0]
    noise = obs_stddev**2
    Kzz = add_jitter(gram(kind, Z, ls, variance), jitter)  # :352-354
    Kzx = cross_covariance(kind, Z, X, ls, variance)  # :355
    Kxx_diag = diagonal(kind, X, ls, variance)  # :356
    mux = np.ones((n, 1)) * mean_const  # :357
    Lz = np.linalg.cholesky(Kzz)  # :359
    A = sla.solve_triangular(Lz, Kzx, lower=True) / np.sqrt(noise)  # :387
    AAT = A @ A.T  # :390
    B = np.eye(m) + AAT  # :393
    L = np.linalg.cholesky(B)  # :396
    log_det_B = 2.0 * np.sum(np.log(np.diagonal(L)))  # :399
    diff = y - mux  # :401
    L_inv_A_diff = sla.solve_triangular(L, A @ diff, lower=True)  # :404
    quad = (np.sum(diff**2) - np.sum(L_inv_A_diff**2)) / noise  # :407
    two_log_prob = -n * np.log(2.0 * np.pi * noise) - log_det_B - quad  # :410
    two_trace = np.sum(Kxx_diag) / noise - np.trace(AAT)  # :413
    return float((two_log_prob - two_trace) / 2.0)  # :416


def sgpr_statistics(kind, X, y, Z, ls, variance, mean_const=0.0) -> dict:
    """The data-dependent sums of the collapsed ELBO over the rows of (X, y):
    P = Kzx Kxz, c = Kzx d, d^T d, sum_i k(x_i, x_i) and the row count.  Sums
    over disjoint row blocks add up to the statistics of their union."""
    X = np.asarray(X, np.float64)
    d = np.asarray(y, np.float64).reshape(-1) - mean_const
    Kzx = cross_covariance(kind, Z, X, ls, variance)
    return {"P": Kzx @ Kzx.T, "c": Kzx @ d, "dd": float(d @ d),
            "kdiag": float(diagonal(kind, X, ls, variance).sum()), "n": X.shape[0]}


def collapsed_elbo_from_statistics(kind, stats, Z, ls, variance, obs_stddev,
                                   jitter=DEFAULT_JITTER) -> float:
    """collapsed_elbo (objectives.py:341-416) from the summed statistics, by the
    reference's algebra: A A^T = Lz^-1 P Lz^-T / s, the quadratic term through
    L^-1 A d = L^-1 Lz^-1 c / sqrt(s) and tr(A A^T) = tr(Lz^-1 P Lz^-T) / s."""
    m = np.asarray(Z).shape[0]
    s = obs_stddev**2
    Kzz = add_jitter(gram(kind, Z, ls, variance), jitter)
    Lz = np.linalg.cholesky(Kzz)
    W = sla.solve_triangular(Lz, sla.solve_triangular(Lz, stats["P"], lower=True).T,
                             lower=True) / s  # A A^T
    L = np.linalg.cholesky(np.eye(m) + W)
    log_det_B = 2.0 * np.sum(np.log(np.diag(L)))
    u = sla.solve_triangular(L, sla.solve_triangular(Lz, stats["c"], lower=True) / np.sqrt(s),
                             lower=True)
    n = stats["n"]
    quad = (stats["dd"] - u @ u) / s
    two_log_prob = -n * np.log(2.0 * np.pi * s) - log_det_B - quad
    two_trace = stats["kdiag"] / s - np.trace(W)
    return float((two_log_prob - two_trace) / 2.0)


def predict(kind, X, y, T, ls, variance, obs_stddev, mean_const=0.0,
            jitter=DEFAULT_JITTER, prior_jitter=DEFAULT_JITTER):
    """ConjugatePosterior.predict (gps.py:494-526); returns (mean [t], cov [t, t])."""
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64).reshape(-1, 1)
    T = np.asarray(T, np.float64)
    n = X.shape[0]
    obs_noise = obs_stddev**2
    mx = np.ones((n, 1)) * mean_const
    Kxx = add_jitter(gram(kind, X, ls, variance), jitter)  # :505-507 (posterior jitter)
    Sigma = Kxx + np.eye(n) * obs_noise  # :509
    L = np.linalg.cholesky(Sigma)  # :511
    mean_t = np.ones((T.shape[0], 1)) * mean_const  # :513
    Ktt = gram(kind, T, ls, variance)  # :514
    Kxt = cross_covariance(kind, X, T, ls, variance)  # :515
    L_inv_Kxt = sla.solve_triangular(L, Kxt, lower=True)  # :517
    L_inv_y_diff = sla.solve_triangular(L, y - mx, lower=True)  # :518
    mean = mean_t + L_inv_Kxt.T @ L_inv_y_diff  # :520
    cov = Ktt - L_inv_Kxt.T @ L_inv_Kxt  # :522
    cov = add_jitter(cov, prior_jitter)  # :523 (prior jitter)
    return np.atleast_1d(mean.squeeze()), cov


def sgpr_predict(kind, X, y, Z, T, ls, variance, obs_stddev, mean_const=0.0,
                 jitter=DEFAULT_JITTER):
    """CollapsedVariationalGaussian.predict (variational_families.py:786-870)."""
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64).reshape(-1, 1)
    Z = np.asarray(Z, np.float64)
    T = np.asarray(T, np.float64)
    m = Z.shape[0]
    noise_var = obs_stddev**2
    Kzx = cross_covariance(kind, Z, X, ls, variance)
    Kzz = add_jitter(gram(kind, Z, ls, variance), jitter)
    Lz = np.linalg.cholesky(Kzz)
    Lz_inv_Kzx = sla.solve_triangular(Lz, Kzx, lower=True)
    A = Lz_inv_Kzx / obs_stddev
    AAT = A @ A.T
    L = np.linalg.cholesky(np.eye(m) + AAT)
    diff = y - mean_const
    Lz_inv_Kzx_diff = sla.cho_solve((L, True), Lz_inv_Kzx @ diff)
    Kzz_inv_Kzx_diff = sla.solve_triangular(Lz.T, Lz_inv_Kzx_diff, lower=False)
    Ktt = gram(kind, T, ls, variance)
    Kzt = cross_covariance(kind, Z, T, ls, variance)
    mut = np.ones((T.shape[0], 1)) * mean_const
    Lz_inv_Kzt = sla.solve_triangular(Lz, Kzt, lower=True)
    L_inv_Lz_inv_Kzt = sla.solve_triangular(L, Lz_inv_Kzt, lower=True)
    mean = mut + (Kzt.T / noise_var) @ Kzz_inv_Kzx_diff
    cov = Ktt - Lz_inv_Kzt.T @ Lz_inv_Kzt + L_inv_Lz_inv_Kzt.T @ L_inv_Lz_inv_Kzt
    cov = add_jitter(cov, jitter)
    return np.atleast_1d(mean.squeeze()), cov


# --------------------------------------------------------------------------
# torch float64 autograd restatement (stand-in for jax.grad of the reference)
# --------------------------------------------------------------------------
def _torch():
    import torch
    return torch


def _t_kernel(kind, x, y, ls, variance):
    torch = _torch()
    xs = x / ls
    ys = y / ls
    sq = ((xs[:, None, :] - ys[None, :, :]) ** 2).sum(-1)
    kind, alpha = _kind(kind)
    if kind == RBF:
        return variance * torch.exp(-0.5 * sq)
    if kind == RATIONAL_QUADRATIC:
        return variance * (1.0 + 0.5 * sq / alpha) ** (-alpha)
    tau = torch.sqrt(torch.clamp(sq, min=_FLOOR))
    if kind == MATERN12:
        return variance * torch.exp(-tau)
    if kind == MATERN32:
        return variance * (1.0 + math.sqrt(3.0) * tau) * torch.exp(-math.sqrt(3.0) * tau)
    return (variance * (1.0 + math.sqrt(5.0) * tau + 5.0 / 3.0 * tau**2)
            * torch.exp(-math.sqrt(5.0) * tau))


def _t_kdiag(kind, x, variance):
    torch = _torch()
    return variance * torch.ones(x.shape[0], dtype=torch.float64)


def _params(ls, variance, obs_stddev, mean_const, d):
    torch = _torch()
    ls_t = torch.tensor(np.asarray(ls, np.float64), requires_grad=True)
    var_t = torch.tensor(float(variance), dtype=torch.float64, requires_grad=True)
    sd_t = torch.tensor(float(obs_stddev), dtype=torch.float64, requires_grad=True)
    c_t = torch.tensor(float(mean_const), dtype=torch.float64, requires_grad=True)
    return ls_t, var_t, sd_t, c_t


def conjugate_mll_torch(kind, X, y, ls, variance, obs_stddev, mean_const=0.0,
                        jitter=DEFAULT_JITTER, lu=True):
    """MLL and its gradient w.r.t. (lengthscale, variance, obs_stddev, constant).

    ``lu=True`` differentiates through slogdet + solve as the reference does
    (operations.py:111,164); ``lu=False`` through a Cholesky factor.
    Returns (value, dict of float64 numpy gradients).
    """
    torch = _torch()
    Xt = torch.as_tensor(np.asarray(X, np.float64))
    yt = torch.as_tensor(np.asarray(y, np.float64).reshape(-1))
    n = Xt.shape[0]
    ls_t, var_t, sd_t, c_t = _params(ls, variance, obs_stddev, mean_const, Xt.shape[1])
    K = _t_kernel(kind, Xt, Xt, ls_t, var_t)
    eye = torch.eye(n, dtype=torch.float64)
    Sigma = K + eye * jitter + eye * sd_t**2
    diff = yt - c_t
    if lu:
        ld = torch.linalg.slogdet(Sigma)[1]
        quad = diff @ torch.linalg.solve(Sigma, diff)
    else:
        L = torch.linalg.cholesky(Sigma)
        ld = 2.0 * torch.log(torch.diagonal(L)).sum()
        z = torch.linalg.solve_triangular(L, diff[:, None], upper=False)[:, 0]
        quad = z @ z
    mll = -0.5 * (n * math.log(2.0 * math.pi) + ld + quad)
    mll.backward()
    grads = {"lengthscale": ls_t.grad.numpy().copy(), "variance": float(var_t.grad),
             "obs_stddev": float(sd_t.grad), "constant": float(c_t.grad)}
    return float(mll.detach()), grads


def conjugate_mll_grad_lu(kind, X, y, ls, variance, obs_stddev, mean_const=0.0,
                          jitter=DEFAULT_JITTER, block=1024):
    """MLL and gradient by the reference's op sequence, lean enough for n = 16384.

    Same quantities as ``conjugate_mll_torch(lu=True)`` without its n x n x d
    autograd graph: Sigma is assembled row block by row block
    (``dense.py:32-36``, ``objectives.py:100-103``); ``slogdet`` and ``solve``
    (``operations.py:111,164``) read one LU factorisation -- the reference
    issues the same LU twice, which XLA's common-subexpression pass merges under
    ``jit`` -- and the gradient is what reverse-mode differentiation of that
    sequence forms: the cotangent of Sigma, 1/2 (alpha alpha^T - Sigma^-1),
    with Sigma^-1 from the LU factors (``solve`` against the identity, as the
    transpose of ``slogdet``'s tangent), contracted block by block with
    dK/dlengthscale and dK/dvariance, plus 2 obs_stddev tr(cotangent) and
    sum(alpha) for the constant mean.  torch float64 on the host's threads.
    Returns (value, dict of float64 numpy gradients) like conjugate_mll_torch.
    """
    torch = _torch()
    Xt = torch.as_tensor(np.asarray(X, np.float64))
    yt = torch.as_tensor(np.asarray(y, np.float64).reshape(-1))
    n, d = Xt.shape
    ls_v = np.broadcast_to(np.asarray(ls, np.float64), (d,)).copy()
    xs = Xt / torch.as_tensor(ls_v)
    s2, sd = float(variance), float(obs_stddev)
    r3, r5 = math.sqrt(3.0), math.sqrt(5.0)

    def sqdist(r0, r1):
        sq = torch.zeros((r1 - r0, n), dtype=torch.float64)
        for k in range(d):  # utils.py:53, one input dimension at a time
            sq += (xs[r0:r1, k, None] - xs[None, :, k]) ** 2
        return sq

    code, ka = _kind(kind)

    def kval(sq):  # unit variance: rbf.py:43, matern32.py:48-53, matern52.py:46-52
        if code == RBF:
            return torch.exp(-0.5 * sq)
        if code == RATIONAL_QUADRATIC:
            return (1.0 + 0.5 * sq / ka) ** (-ka)
        tau = torch.sqrt(torch.clamp(sq, min=_FLOOR))
        if code == MATERN12:
            return torch.exp(-tau)
        if code == MATERN32:
            return (1.0 + r3 * tau) * torch.exp(-r3 * tau)
        return (1.0 + r5 * tau + 5.0 / 3.0 * tau * tau) * torch.exp(-r5 * tau)

    def dcoef(sq):  # dk/dl_k = s2 * dcoef * (x_k - y_k)^2 / l_k^3 (zero below the floor)
        if code == RBF:
            return torch.exp(-0.5 * sq)
        if code == RATIONAL_QUADRATIC:
            return (1.0 + 0.5 * sq / ka) ** (-ka - 1.0)
        tau = torch.sqrt(torch.clamp(sq, min=_FLOOR))
        if code == MATERN12:
            c = torch.exp(-tau) / tau
        elif code == MATERN32:
            c = 3.0 * torch.exp(-r3 * tau)
        else:
            c = 5.0 / 3.0 * (1.0 + r5 * tau) * torch.exp(-r5 * tau)
        return torch.where(sq > _FLOOR, c, torch.zeros_like(c))

    Sigma = torch.empty((n, n), dtype=torch.float64)
    for r0 in range(0, n, block):
        r1 = min(n, r0 + block)
        Sigma[r0:r1] = s2 * kval(sqdist(r0, r1))
    Sigma.diagonal().add_(jitter).add_(sd * sd)
    diff = yt - float(mean_const)
    LU, piv = torch.linalg.lu_factor(Sigma)
    logdet = torch.log(torch.abs(torch.diagonal(LU))).sum()
    alpha = torch.linalg.lu_solve(LU, piv, diff[:, None])[:, 0]
    mll = -0.5 * (n * math.log(2.0 * math.pi) + float(logdet) + float(diff @ alpha))
    del Sigma
    W = torch.linalg.lu_solve(LU, piv, torch.eye(n, dtype=torch.float64))  # Sigma^-1
    del LU
    g_ls = np.zeros(d)
    g_var = 0.0
    for r0 in range(0, n, block):
        r1 = min(n, r0 + block)
        sq = sqdist(r0, r1)
        G = 0.5 * (alpha[r0:r1, None] * alpha[None, :] - W[r0:r1])  # cotangent of Sigma
        g_var += float((G * kval(sq)).sum())
        Gc = G * dcoef(sq)
        for k in range(d):
            g_ls[k] += s2 * float((Gc * (xs[r0:r1, k, None] - xs[None, :, k]) ** 2).sum()) / ls_v[k]
    g_noise = 0.5 * float((alpha * alpha).sum() - torch.diagonal(W).sum())
    ls_grad = np.array(g_ls.sum()) if np.ndim(ls) == 0 else g_ls
    grads = {"lengthscale": ls_grad, "variance": g_var, "obs_stddev": 2.0 * sd * g_noise,
             "constant": float(alpha.sum())}
    return mll, grads


def collapsed_elbo_torch(kind, X, y, Z, ls, variance, obs_stddev, mean_const=0.0,
                         jitter=DEFAULT_JITTER):
    """collapsed_elbo and gradients w.r.t. (lengthscale, variance, obs_stddev,
    constant, inducing_inputs), same op order as objectives.py:341-416."""
    torch = _torch()
    Xt = torch.as_tensor(np.asarray(X, np.float64))
    yt = torch.as_tensor(np.asarray(y, np.float64).reshape(-1, 1))
    Zt = torch.tensor(np.asarray(Z, np.float64), requires_grad=True)
    n, m = Xt.shape[0], Zt.shape[0]
    ls_t, var_t, sd_t, c_t = _params(ls, variance, obs_stddev, mean_const, Xt.shape[1])
    noise = sd_t**2
    Kzz = _t_kernel(kind, Zt, Zt, ls_t, var_t) + torch.eye(m, dtype=torch.float64) * jitter
    Kzx = _t_kernel(kind, Zt, Xt, ls_t, var_t)
    Kxx_diag = _t_kdiag(kind, Xt, var_t)
    Lz = torch.linalg.cholesky(Kzz)
    A = torch.linalg.solve_triangular(Lz, Kzx, upper=False) / torch.sqrt(noise)
    AAT = A @ A.T
    B = torch.eye(m, dtype=torch.float64) + AAT
    L = torch.linalg.cholesky(B)
    log_det_B = 2.0 * torch.log(torch.diagonal(L)).sum()
    diff = yt - c_t
    LiAd = torch.linalg.solve_triangular(L, A @ diff, upper=False)
    quad = ((diff**2).sum() - (LiAd**2).sum()) / noise
    two_log_prob = -n * torch.log(2.0 * math.pi * noise) - log_det_B - quad
    two_trace = Kxx_diag.sum() / noise - torch.trace(AAT)
    elbo = (two_log_prob - two_trace) / 2.0
    elbo.backward()
    grads = {"lengthscale": ls_t.grad.numpy().copy(), "variance": float(var_t.grad),
             "obs_stddev": float(sd_t.grad), "constant": float(c_t.grad),
             "inducing_inputs": Zt.grad.numpy().copy()}
    return float(elbo.detach()), grads


def central_fd(f, x0: np.ndarray, h: float = 1e-5) -> np.ndarray:
    """Central finite differences of scalar f at x0 (relative step h*max(1,|x|))."""
    x0 = np.asarray(x0, np.float64)
    g = np.zeros_like(x0)
    for i in range(x0.size):
        e = np.zeros_like(x0)
        step = h * max(1.0, abs(x0.flat[i]))
        e.flat[i] = step
        g.flat[i] = (f(x0 + e) - f(x0 - e)) / (2 * step)
    return g
