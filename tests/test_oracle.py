"""CPU: the float64 oracle against the reference's own known answers and
identities (the oracle is the checker for every GPU parity test)."""
import numpy as np
import pytest
import scipy.stats

from oracle import gp_oracle as O


def _data(n, d, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-2.0, 2.0, size=(n, d))
    y = np.sin(x[:, :1]) + 0.1 * rng.standard_normal((n, 1))
    return x, y


def test_linalg_known_answers():
    # tests/test_linalg.py:330-348 and :380-396 of the reference
    A = np.array([[2.0, 1.0], [1.0, 3.0]])
    b = np.array([1.0, 2.0])
    assert np.allclose(A @ O.solve_dense(A, b), b)
    assert np.isclose(O.logdet_dense(A), np.log(5.0))
    L = np.array([[2.0, 0.0], [1.0, 3.0]])
    assert np.isclose(np.sum(np.log(np.diag(L))), np.log(6.0))
    Lc = np.linalg.cholesky(A)
    assert np.allclose(Lc @ Lc.T, A, atol=1e-6)


@pytest.mark.parametrize("n", [1, 2, 5, 100])
def test_log_prob_matches_mvn(n):
    # tests/test_gaussian_distribution.py:102-123: Dense log_prob == MVN log_prob
    rng = np.random.default_rng(n)
    mean = rng.uniform(size=n)
    sq = rng.uniform(size=(n, n))
    cov = sq @ sq.T + 1e-3 * np.eye(n)
    y = rng.uniform(size=n)
    ref = scipy.stats.multivariate_normal(mean, cov).logpdf(y)
    assert np.isclose(O.gaussian_log_prob(mean, cov, y), ref, rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("n_points", [10, 20])
@pytest.mark.parametrize("n_dims", [1, 2, 3])
@pytest.mark.parametrize("seed", [123, 42])
def test_collapsed_elbo_equals_mll_when_z_is_x(n_points, n_dims, seed):
    # tests/test_objectives.py:193-199: with Z = X the bound is tight
    x, y = _data(n_points, n_dims, seed)
    mll = O.conjugate_mll(O.RBF, x, y, 1.0, 1.0, 1.0, 0.0)
    elbo = O.collapsed_elbo(O.RBF, x, y, x, 1.0, 1.0, 1.0, 0.0)
    assert abs(elbo - mll) / abs(mll) < 1e-6


@pytest.mark.parametrize("kind", [O.RBF, O.MATERN32, O.MATERN52])
def test_lu_and_cholesky_forms_agree(kind):
    x, y = _data(50, 3, 0)
    ls = np.array([0.5, 1.0, 2.0])
    a = O.conjugate_mll(kind, x, y, ls, 1.3, 0.2, 0.1)
    b = O.conjugate_mll_cholesky(kind, x, y, ls, 1.3, 0.2, 0.1)
    assert abs(a - b) <= 1e-10 * abs(a)


@pytest.mark.parametrize("kind", [O.RBF, O.MATERN32, O.MATERN52])
def test_mll_gradient_vs_finite_differences(kind):
    x, y = _data(30, 2, 1)
    ls, var, sd, c = np.array([0.7, 1.4]), 1.2, 0.3, 0.05
    val, g = O.conjugate_mll_torch(kind, x, y, ls, var, sd, c)
    assert np.isclose(val, O.conjugate_mll(kind, x, y, ls, var, sd, c), rtol=1e-12)
    _, g_chol = O.conjugate_mll_torch(kind, x, y, ls, var, sd, c, lu=False)
    vec = np.concatenate([ls, [var, sd, c]])

    def f(v):
        return O.conjugate_mll(kind, x, y, v[:2], v[2], v[3], v[4])
    fd = O.central_fd(f, vec, 1e-6)
    ad = np.concatenate([g["lengthscale"], [g["variance"], g["obs_stddev"], g["constant"]]])
    adc = np.concatenate([g_chol["lengthscale"],
                          [g_chol["variance"], g_chol["obs_stddev"], g_chol["constant"]]])
    assert np.allclose(ad, fd, rtol=1e-5, atol=1e-6)
    assert np.allclose(ad, adc, rtol=1e-10, atol=1e-10)


def test_elbo_gradient_vs_finite_differences():
    rng = np.random.default_rng(3)
    x, y = _data(40, 2, 3)
    z = rng.uniform(-2, 2, size=(7, 2))
    ls, var, sd = np.array([0.8, 1.1]), 0.9, 0.25
    val, g = O.collapsed_elbo_torch(O.RBF, x, y, z, ls, var, sd, 0.0)
    assert np.isclose(val, O.collapsed_elbo(O.RBF, x, y, z, ls, var, sd, 0.0), rtol=1e-12)
    fz = O.central_fd(lambda zz: O.collapsed_elbo(O.RBF, x, y, zz.reshape(7, 2), ls, var, sd),
                      z.reshape(-1), 1e-6)
    assert np.allclose(g["inducing_inputs"].reshape(-1), fz, rtol=1e-4, atol=1e-6)


def test_predict_matches_direct_formula():
    x, y = _data(40, 2, 5)
    t = np.random.default_rng(9).uniform(-2, 2, size=(11, 2))
    mean, cov = O.predict(O.MATERN52, x, y, t, 0.9, 1.1, 0.3, 0.2)
    S = O.gram(O.MATERN52, x, 0.9, 1.1) + (1e-6 + 0.09) * np.eye(40)
    Kxt = O.cross_covariance(O.MATERN52, x, t, 0.9, 1.1)
    mean2 = 0.2 + Kxt.T @ np.linalg.solve(S, y[:, 0] - 0.2)
    cov2 = O.gram(O.MATERN52, t, 0.9, 1.1) - Kxt.T @ np.linalg.solve(S, Kxt) + 1e-6 * np.eye(11)
    assert np.allclose(mean, mean2, rtol=1e-10, atol=1e-10)
    assert np.allclose(cov, cov2, rtol=1e-9, atol=1e-10)


def test_golden_fixtures_reproduce():
    """The committed fixtures (tests/golden) still match the oracle."""
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "golden_small.npz")
    g = np.load(path)
    for case in range(int(g["ncases"])):
        p = lambda k: g[f"c{case}_{k}"]  # noqa: E731
        kind = int(p("kind"))
        val = O.conjugate_mll(kind, p("x"), p("y"), p("ls"), float(p("var")), float(p("sd")),
                              float(p("c")))
        assert np.isclose(val, float(p("mll")), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("kind,nu", [(O.RBF, None), (O.MATERN32, 1.5), (O.MATERN52, 2.5)])
@pytest.mark.parametrize("ard", [True, False])
def test_kernel_values_match_an_independent_implementation(kind, nu, ard):
    """The oracle's stationary kernels (kernels/stationary/rbf.py:40-44,
    matern32.py:41-54, matern52.py:42-53 of the reference) against
    scikit-learn's RBF / Matern on the same scaled Euclidean distance."""
    gpk = pytest.importorskip("sklearn.gaussian_process.kernels")
    rng = np.random.default_rng(7)
    x, y = rng.standard_normal((40, 3)), rng.standard_normal((30, 3))
    ls = np.array([0.4, 1.1, 2.5]) if ard else 0.8
    var = 1.7
    base = gpk.RBF(length_scale=ls) if nu is None else gpk.Matern(length_scale=ls, nu=nu)
    ref = (gpk.ConstantKernel(var) * base)(x, y)
    assert np.allclose(O.cross_covariance(kind, x, y, ls, var), ref, rtol=1e-12, atol=1e-14)
    K = O.gram(kind, x, ls, var)
    assert np.allclose(K, (gpk.ConstantKernel(var) * base)(x), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("kind,nu", [(O.RBF, None), (O.MATERN32, 1.5), (O.MATERN52, 2.5)])
def test_mll_matches_an_independent_implementation(kind, nu):
    """The oracle's conjugate_mll and its gradient against scikit-learn's
    Gaussian-process log marginal likelihood (zero mean, Sigma = var K +
    (obs_stddev^2 + jitter) I); scikit-learn differentiates in log
    hyperparameters, so d/dlog(l) = l d/dl and d/dlog(var) = var d/dvar."""
    gpk = pytest.importorskip("sklearn.gaussian_process.kernels")
    gpr_mod = pytest.importorskip("sklearn.gaussian_process")
    rng = np.random.default_rng(11)
    n, d = 60, 3
    x = rng.uniform(-2, 2, size=(n, d))
    y = (np.sin(x).sum(1) + 0.1 * rng.standard_normal(n))[:, None]
    ls, var, sd, jitter = np.array([0.6, 1.3, 2.2]), 1.4, 0.3, 1e-6
    base = gpk.RBF(length_scale=ls) if nu is None else gpk.Matern(length_scale=ls, nu=nu)
    kern = gpk.ConstantKernel(var) * base
    gpr = gpr_mod.GaussianProcessRegressor(kernel=kern, alpha=sd * sd + jitter, optimizer=None,
                                           normalize_y=False).fit(x, y[:, 0])
    lml, dlml = gpr.log_marginal_likelihood(gpr.kernel_.theta, eval_gradient=True)
    val = O.conjugate_mll(kind, x, y, ls, var, sd, 0.0, jitter=jitter)
    assert abs(val - lml) <= 1e-10 * abs(lml)
    _, g = O.conjugate_mll_torch(kind, x, y, ls, var, sd, 0.0, lu=False)
    # scikit-learn's theta: [log var, log l_1 .. log l_d]
    assert np.isclose(dlml[0], var * g["variance"], rtol=1e-8)
    assert np.allclose(dlml[1:], ls * np.asarray(g["lengthscale"]), rtol=1e-8)


@pytest.mark.parametrize("kind,nu", [(O.RBF, None), (O.MATERN52, 2.5)])
def test_predict_matches_an_independent_implementation(kind, nu):
    """The oracle's ConjugatePosterior.predict against scikit-learn's posterior
    mean and covariance (alpha = obs_stddev^2 + posterior jitter; the oracle
    adds the prior's jitter to the predictive covariance, gps.py:523)."""
    gpk = pytest.importorskip("sklearn.gaussian_process.kernels")
    gpr_mod = pytest.importorskip("sklearn.gaussian_process")
    rng = np.random.default_rng(13)
    x = rng.uniform(-2, 2, size=(80, 2))
    y = (np.sin(2 * x).sum(1) + 0.1 * rng.standard_normal(80))[:, None]
    t = rng.uniform(-2.5, 2.5, size=(25, 2))
    ls, var, sd, jit, pjit = np.array([0.7, 1.2]), 1.1, 0.2, 1e-6, 1e-5
    base = gpk.RBF(length_scale=ls) if nu is None else gpk.Matern(length_scale=ls, nu=nu)
    gpr = gpr_mod.GaussianProcessRegressor(kernel=gpk.ConstantKernel(var) * base,
                                           alpha=sd * sd + jit, optimizer=None,
                                           normalize_y=False).fit(x, y[:, 0])
    m_ref, c_ref = gpr.predict(t, return_cov=True)
    mean, cov = O.predict(kind, x, y, t, ls, var, sd, 0.0, jitter=jit, prior_jitter=pjit)
    assert np.allclose(mean, m_ref, rtol=1e-9, atol=1e-10)
    assert np.allclose(cov - pjit * np.eye(len(t)), c_ref, rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize("kind", [O.RBF, O.MATERN32, O.MATERN52])
@pytest.mark.parametrize("m", [5, 25])
def test_collapsed_elbo_matches_the_textbook_form(kind, m):
    """The oracle follows the reference's op sequence (objectives.py:341-416:
    A = Lz^-1 Kzx / sqrt(s), B = I + A A^T); here the same bound from its
    closed form log N(y; mean, Q + s I) - tr(Kxx - Q) / (2 s), Q = Kxz Kzz^-1 Kzx,
    evaluated densely -- an independent formula for the same quantity."""
    rng = np.random.default_rng(m + kind)
    n, d = 70, 2
    x = rng.uniform(-2, 2, size=(n, d))
    y = (np.sin(x).sum(1) + 0.1 * rng.standard_normal(n))[:, None]
    z = x[rng.choice(n, m, replace=False)] + 0.05 * rng.standard_normal((m, d))
    ls, var, sd, c, jit = np.array([0.8, 1.3]), 1.2, 0.3, 0.1, 1e-6
    s = sd * sd
    Kzz = O.gram(kind, z, ls, var) + jit * np.eye(m)
    Kxz = O.cross_covariance(kind, x, z, ls, var)
    Q = Kxz @ np.linalg.solve(Kzz, Kxz.T)
    ref = scipy.stats.multivariate_normal(np.full(n, c), Q + s * np.eye(n)).logpdf(y[:, 0])
    ref -= (np.sum(O.diagonal(kind, x, ls, var)) - np.trace(Q)) / (2 * s)
    got = O.collapsed_elbo(kind, x, y, z, ls, var, sd, c, jitter=jit)
    assert abs(got - ref) <= 1e-9 * abs(ref), (got, ref)


@pytest.mark.parametrize("kind", [O.RBF, O.MATERN32, O.MATERN52])
@pytest.mark.parametrize("ard", [True, False])
def test_lean_lu_port_matches_autograd(kind, ard):
    """The row-blocked port that times the reference's algorithm at n = 16384
    gives the autograd value and gradient of the same LU op sequence."""
    rng = np.random.default_rng(7 + kind)
    n, d = 300, 3
    x = rng.standard_normal((n, d))
    y = rng.standard_normal((n, 1))
    ls = np.exp(rng.uniform(-1, 1, d)) if ard else np.array(1.3)
    v1, g1 = O.conjugate_mll_torch(kind, x, y, ls, 1.2, 0.3, 0.1)
    v2, g2 = O.conjugate_mll_grad_lu(kind, x, y, ls, 1.2, 0.3, 0.1, block=128)
    a = np.concatenate([np.atleast_1d(g1["lengthscale"]),
                        [g1["variance"], g1["obs_stddev"], g1["constant"]]])
    b = np.concatenate([np.atleast_1d(g2["lengthscale"]),
                        [g2["variance"], g2["obs_stddev"], g2["constant"]]])
    assert abs(v1 - v2) <= 1e-12 * abs(v1)
    assert np.allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(a).max())


@pytest.mark.parametrize("ard", [True, False])
def test_matern12_and_rational_quadratic_match_an_independent_implementation(ard):
    """Matern12 (matern12.py:44-48) against scikit-learn's Matern(nu=0.5), and the
    isotropic RationalQuadratic (rational_quadratic.py:76-83) against
    scikit-learn's RationalQuadratic (scalar length scale only)."""
    gpk = pytest.importorskip("sklearn.gaussian_process.kernels")
    rng = np.random.default_rng(9)
    x, y = rng.standard_normal((40, 3)), rng.standard_normal((30, 3))
    ls = np.array([0.4, 1.1, 2.5]) if ard else 0.8
    ref = (gpk.ConstantKernel(1.7) * gpk.Matern(length_scale=ls, nu=0.5))(x, y)
    assert np.allclose(O.cross_covariance(O.MATERN12, x, y, ls, 1.7), ref, rtol=1e-12, atol=1e-14)
    if not ard:
        for alpha in (0.5, 2.0):
            ref = (gpk.ConstantKernel(1.7) * gpk.RationalQuadratic(length_scale=ls, alpha=alpha))(x, y)
            got = O.cross_covariance(O.rational_quadratic(alpha), x, y, ls, 1.7)
            assert np.allclose(got, ref, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("kind", [O.MATERN12, O.rational_quadratic(0.7)])
@pytest.mark.parametrize("ard", [True, False])
def test_added_kernels_lean_port_and_finite_differences(kind, ard):
    """The lean port and autograd agree for the added kernels, and both match
    central differences of the value."""
    rng = np.random.default_rng(21)
    n, d = 120, 3
    x = rng.standard_normal((n, d))
    y = rng.standard_normal((n, 1))
    ls = np.exp(rng.uniform(-0.5, 0.5, d)) if ard else np.array(1.1)
    v1, g1 = O.conjugate_mll_torch(kind, x, y, ls, 1.2, 0.3, 0.1)
    v2, g2 = O.conjugate_mll_grad_lu(kind, x, y, ls, 1.2, 0.3, 0.1, block=64)
    a = np.concatenate([np.atleast_1d(g1["lengthscale"]),
                        [g1["variance"], g1["obs_stddev"], g1["constant"]]])
    b = np.concatenate([np.atleast_1d(g2["lengthscale"]),
                        [g2["variance"], g2["obs_stddev"], g2["constant"]]])
    assert abs(v1 - v2) <= 1e-12 * abs(v1)
    assert np.allclose(a, b, rtol=1e-10, atol=1e-10 * np.abs(a).max())
    vec = np.concatenate([np.atleast_1d(ls), [1.2, 0.3, 0.1]])
    nl = vec.size - 3

    def f(v):
        lsv = v[:nl] if ard else np.array(v[0])
        return O.conjugate_mll(kind, x, y, lsv, v[nl], v[nl + 1], v[nl + 2])
    fd = O.central_fd(f, vec, 1e-6)
    assert np.allclose(a, fd, rtol=1e-5, atol=1e-6 * np.abs(fd).max())


@pytest.mark.parametrize("kind", [O.RBF, O.MATERN52])
def test_loocv_oracle_gradient_and_identity(kind):
    """conjugate_loocv's autograd gradient matches central differences, and the
    value equals the explicit leave-one-out sum (refit without point i, predict it)."""
    rng = np.random.default_rng(5)
    n, d = 25, 2
    x = rng.uniform(-2, 2, (n, d))
    y = (np.sin(x).sum(1) + 0.1 * rng.standard_normal(n))[:, None]
    ls, var, sd, c = np.array([0.8, 1.3]), 1.1, 0.3, 0.2
    v, g = O.conjugate_loocv_torch(kind, x, y, ls, var, sd, c)
    assert abs(v - O.conjugate_loocv(kind, x, y, ls, var, sd, c)) < 1e-10 * abs(v)
    vec = np.concatenate([ls, [var, sd, c]])
    fd = O.central_fd(lambda p: O.conjugate_loocv(kind, x, y, p[:2], p[2], p[3], p[4]), vec, 1e-6)
    gv = np.concatenate([g["lengthscale"], [g["variance"], g["obs_stddev"], g["constant"]]])
    assert np.allclose(gv, fd, rtol=1e-5, atol=1e-7)
    # brute force: for each i, the predictive density of y_i from the other n-1 points
    S = O.gram(kind, x, ls, var) + np.eye(n) * (sd * sd + 1e-6)
    tot = 0.0
    for i in range(n):
        keep = np.arange(n) != i
        Sk = S[np.ix_(keep, keep)]
        kv = S[i, keep]
        w = np.linalg.solve(Sk, kv)
        mu = c + w @ (y[keep, 0] - c)
        var_i = S[i, i] - kv @ w
        tot += -0.5 * np.log(2 * np.pi * var_i) - 0.5 * (y[i, 0] - mu) ** 2 / var_i
    assert abs(tot - v) < 1e-9 * abs(v)
