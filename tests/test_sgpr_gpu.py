"""GPU parity of collapsed_elbo (value, gradients w.r.t. kernel, likelihood and
mean parameters and the inducing inputs), of the cross-covariance cotangent and
of the SGPR predictive, against the float64 oracle / torch float64 autograd."""
import numpy as np
import pytest
import torch

import gpjax_gb300 as gpx
from oracle import gp_oracle as O
from tests._gpu_helpers import KINDS

pytestmark = pytest.mark.gpu


def _family(kind, Z, ls, var, sd, c, jitter=1e-6):
    kern = KINDS[kind](lengthscale=np.asarray(ls, np.float64), variance=var)
    prior = gpx.gps.Prior(kernel=kern, mean_function=gpx.mean_functions.Constant(
        gpx.parameters.Real(c)))
    post = prior * gpx.likelihoods.Gaussian(num_datapoints=1, obs_stddev=sd)
    q = gpx.variational_families.CollapsedVariationalGaussian(post, Z, jitter=jitter)
    for p in (kern.lengthscale, kern.variance, post.likelihood.obs_stddev,
              prior.mean_function.constant, q.inducing_inputs):
        p.to("cuda").requires_grad_(True)
    return q


def _run(kind, x, y, Z, ls, var, sd, c, precision="fp64"):
    q = _family(kind, Z, ls, var, sd, c)
    val = gpx.objectives.collapsed_elbo(q, gpx.Dataset(X=x, y=y), precision=precision)
    val.backward()
    k = q.posterior.prior.kernel
    g = np.concatenate([np.atleast_1d(k.lengthscale.value.grad.cpu().numpy()),
                        [float(k.variance.value.grad),
                         float(q.posterior.likelihood.obs_stddev.value.grad),
                         float(q.posterior.prior.mean_function.constant.value.grad)]])
    return float(val.detach()), g, q.inducing_inputs.value.grad.cpu().numpy()


def _oracle(kind, x, y, Z, ls, var, sd, c):
    val, g = O.collapsed_elbo_torch(kind, x, y, Z, ls, var, sd, c)
    gv = np.concatenate([np.atleast_1d(g["lengthscale"]),
                         [g["variance"], g["obs_stddev"], g["constant"]]])
    return val, gv, g["inducing_inputs"]


@pytest.mark.parametrize("kind,n,m,d,ard", [(0, 50, 7, 1, False), (1, 300, 20, 2, True),
                                            (2, 1000, 64, 3, True), (0, 9000, 100, 8, True),
                                            (2, 700, 130, 5, False)])
def test_collapsed_elbo_fp64(cuda_lib, kind, n, m, d, ard):
    rng = np.random.default_rng(n + m)
    x = rng.uniform(-2, 2, size=(n, d))
    y = np.sin(x).sum(1, keepdims=True) + 0.1 * rng.standard_normal((n, 1))
    if d == 1:  # spread inducing points: well-conditioned Kzz for a gradient check
        Z = np.linspace(-2, 2, m)[:, None]
    else:
        Z = x[rng.choice(n, m, replace=False)] + 0.05 * rng.standard_normal((m, d))
    ls = np.exp(rng.uniform(np.log(0.5), np.log(2.0), d)) if ard else np.array(1.1)
    val, g, gz = _run(kind, x, y, Z, ls, 1.2, 0.3, 0.1)
    ref, gref, gzref = _oracle(kind, x, y, Z, ls, 1.2, 0.3, 0.1)
    # float64 forward error grows with cond(Kzz): the library forms K^-1 and
    # Su^-1 explicitly, the reference solves through Lz; both are float64-exact
    # up to ~cond * eps
    cond = np.linalg.cond(O.gram(kind, Z, ls, 1.2) + 1e-6 * np.eye(m))
    tol = max(1e-9, 1e-12 * cond)
    assert abs(val - ref) <= tol * abs(ref), (val, ref, cond)
    assert np.allclose(g, gref, rtol=max(1e-6, 10 * tol), atol=1e-7 * np.abs(gref).max()), (g, gref)
    assert np.allclose(gz, gzref, rtol=max(1e-6, 10 * tol), atol=1e-7 * np.abs(gzref).max())


@pytest.mark.parametrize("n_points", [10, 20])
@pytest.mark.parametrize("n_dims", [1, 2, 3])
def test_collapsed_elbo_equals_mll_when_z_is_x(cuda_lib, n_points, n_dims):
    # tests/test_objectives.py:193-199 of the reference
    rng = np.random.default_rng(n_points * 10 + n_dims)
    x = rng.uniform(-2, 2, size=(n_points, n_dims))
    y = np.sin(x[:, :1]) + 0.1 * rng.standard_normal((n_points, 1))
    q = _family(0, x, np.ones(n_dims), 1.0, 1.0, 0.0)
    elbo = float(gpx.objectives.collapsed_elbo(q, gpx.Dataset(X=x, y=y), precision="fp64"))
    mll = float(gpx.objectives.conjugate_mll(q.posterior, gpx.Dataset(X=x, y=y), precision="fp64"))
    assert abs(elbo - mll) / abs(mll) < 1e-6


def test_collapsed_elbo_mixed(cuda_lib):
    """Mixed form (float32 Phi, float64 m x m algebra) on a mixture-of-Gaussians
    input like the SGPR workload, at reduced n; errors are reported."""
    rng = np.random.default_rng(5)
    n, m, d = 20000, 128, 8
    means = rng.uniform(-5, 5, size=(16, d))
    x = means[rng.integers(0, 16, n)] + 0.5 * rng.standard_normal((n, d))
    y = np.sin(x).sum(1, keepdims=True) + 0.1 * rng.standard_normal((n, 1))
    Z = x[rng.choice(n, m, replace=False)]
    ls = np.exp(rng.uniform(np.log(0.5), np.log(2.0), d))
    v64, g64, z64 = _run(0, x, y, Z, ls, 1.0, 0.1, 0.0, "fp64")
    vm, gm, zm = _run(0, x, y, Z, ls, 1.0, 0.1, 0.0, "mixed")
    ref = O.collapsed_elbo(0, x, y, Z, ls, 1.0, 0.1, 0.0)
    print(f"SGPR n={n} m={m}: fp64 rel {abs(v64 - ref) / abs(ref):.2e}, "
          f"mixed rel {abs(vm - ref) / abs(ref):.2e}, "
          f"mixed grad rel {np.linalg.norm(gm - g64) / np.linalg.norm(g64):.2e}")
    assert abs(v64 - ref) <= 1e-9 * abs(ref)
    assert abs(vm - ref) <= 1e-4 * abs(ref)
    assert np.linalg.norm(gm - g64) <= 1e-2 * np.linalg.norm(g64)


@pytest.mark.parametrize("kind,n,m,d,vtol,ztol", [
    (0, 20000, 128, 8, 1e-5, 2e-3),   # wide adjoint tiles (n >= 2048, d <= 8)
    (2, 1500, 70, 3, 1e-5, 2e-3),     # narrow adjoint tiles, ragged m
    (1, 5000, 300, 12, 1e-5, 2e-3),   # narrow tiles with the 16-wide input bound
    # wide tiles for P (two n-chunks, the last ragged); 1024 inducing points in
    # 8 tight clusters: the Z gradient is a difference of its Phi and Kzz parts
    # (norms ~5e3 and ~4.5e3 against ~1.8e3) and moves by ~1e-2 for a random
    # 1e-7 relative error in P, which float32 accumulation of P already makes
    # (CPU emulation with float32 chunks of P: 9.5e-3)
    (0, 9000, 1024, 8, 2e-5, 5e-2),
])
def test_collapsed_elbo_mixed_tensor_core(cuda_lib, kind, n, m, d, vtol, ztol):
    """Mixed form (Phi in TF32 hi/lo, P and the Phi adjoint on the tensor cores,
    float64 m x m algebra) against the float64 form on the same inputs."""
    rng = np.random.default_rng(n + m + d)
    means = rng.uniform(-3, 3, size=(8, d))
    x = means[rng.integers(0, 8, n)] + 0.5 * rng.standard_normal((n, d))
    y = np.sin(x).sum(1, keepdims=True) + 0.1 * rng.standard_normal((n, 1))
    Z = x[rng.choice(n, m, replace=False)]
    ls = np.exp(rng.uniform(np.log(0.7), np.log(2.0), d))
    v64, g64, z64 = _run(kind, x, y, Z, ls, 1.1, 0.2, 0.05, "fp64")
    vm, gm, zm = _run(kind, x, y, Z, ls, 1.1, 0.2, 0.05, "mixed")
    ev = abs(vm - v64) / abs(v64)
    eg = np.linalg.norm(gm - g64) / np.linalg.norm(g64)
    ez = np.linalg.norm(zm - z64) / np.linalg.norm(z64)
    print(f"SGPR mixed kind={kind} n={n} m={m} d={d}: value {ev:.2e}, theta grad {eg:.2e}, "
          f"Z grad {ez:.2e}")
    assert ev <= vtol
    assert eg <= 1e-3
    assert ez <= ztol


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("ard", [True, False])
def test_cross_covariance_vjp(cuda_lib, kind, ard):
    rng = np.random.default_rng(kind)
    n, m, d = 37, 29, 3
    x, y = rng.standard_normal((n, d)), rng.standard_normal((m, d)) + 0.3
    W = rng.standard_normal((n, m))
    ls = np.array([0.6, 1.1, 1.7]) if ard else np.array(0.9)
    k = KINDS[kind](lengthscale=ls, variance=1.3)
    k.lengthscale.to("cuda").requires_grad_(True)
    k.variance.to("cuda").requires_grad_(True)
    X = torch.tensor(x, device="cuda", requires_grad=True)
    Y = torch.tensor(y, device="cuda", requires_grad=True)
    (k.cross_covariance(X, Y) * torch.as_tensor(W, device="cuda")).sum().backward()
    # torch float64 autograd of the oracle kernel
    lt = torch.tensor(ls, requires_grad=True)
    vt = torch.tensor(1.3, dtype=torch.float64, requires_grad=True)
    xt = torch.tensor(x, requires_grad=True)
    yt = torch.tensor(y, requires_grad=True)
    (O._t_kernel(kind, xt, yt, lt, vt) * torch.as_tensor(W)).sum().backward()
    assert np.allclose(k.lengthscale.value.grad.cpu().numpy(), lt.grad.numpy(), rtol=1e-10)
    assert np.isclose(float(k.variance.value.grad), float(vt.grad), rtol=1e-10)
    assert np.allclose(X.grad.cpu().numpy(), xt.grad.numpy(), rtol=1e-9, atol=1e-12)
    assert np.allclose(Y.grad.cpu().numpy(), yt.grad.numpy(), rtol=1e-9, atol=1e-12)


def test_sgpr_predict(cuda_lib):
    rng = np.random.default_rng(2)
    n, m, t, d = 400, 30, 25, 2
    x = rng.uniform(-2, 2, size=(n, d))
    y = np.sin(x).sum(1, keepdims=True) + 0.1 * rng.standard_normal((n, 1))
    Z = x[:m].copy()
    T = rng.uniform(-2, 2, size=(t, d))
    q = _family(2, Z, np.array([0.8, 1.2]), 1.1, 0.2, 0.05)
    dist = q.predict(torch.as_tensor(T, device="cuda"), gpx.Dataset(X=x, y=y))
    mean, cov = O.sgpr_predict(2, x, y, Z, T, np.array([0.8, 1.2]), 1.1, 0.2, 0.05)
    assert np.allclose(dist.mean.cpu().numpy(), mean, rtol=1e-8, atol=1e-9)
    assert np.allclose(dist.covariance().cpu().numpy(), cov, rtol=1e-7, atol=1e-9)


def test_collapsed_elbo_fp64_ill_conditioned_value(cuda_lib):
    """Near-duplicate inducing points (cond(Kzz) ~ 3e6): the value still agrees
    to ~cond * eps."""
    rng = np.random.default_rng(57)
    n, m, d = 50, 7, 1
    x = rng.uniform(-2, 2, size=(n, d))
    y = np.sin(x).sum(1, keepdims=True) + 0.1 * rng.standard_normal((n, 1))
    Z = x[rng.choice(n, m, replace=False)] + 0.05 * rng.standard_normal((m, d))
    ls = np.array(1.1)
    q = _family(0, Z, ls, 1.2, 0.3, 0.1)
    val = float(gpx.objectives.collapsed_elbo(q, gpx.Dataset(X=x, y=y), precision="fp64"))
    ref = O.collapsed_elbo(0, x, y, Z, ls, 1.2, 0.3, 0.1)
    cond = np.linalg.cond(O.gram(0, Z, ls, 1.2) + 1e-6 * np.eye(m))
    assert abs(val - ref) <= max(1e-9, 1e-12 * cond) * abs(ref), (val, ref, cond)


@pytest.mark.parametrize("precision,vtol,gtol", [("fp64", 1e-9, 1e-7), ("mixed", 1e-5, 2e-3)])
def test_sharded_elbo_two_ranks_match_single(cuda_lib, precision, vtol, gtol):
    """gpk_collapsed_elbo_sharded as two ranks -- two host threads, each on its
    own stream with half the rows, exchanging through a host-side sum in the
    callback (the device never waits on the other rank) -- against one
    float64 gpk_collapsed_elbo call on all rows: the float64 form to 1e-9
    (summation order differs), the mixed form at the mixed SGPR tolerances."""
    import threading

    from gpjax_gb300 import _lib
    from gpjax_gb300.objectives import shard_rows
    lib = _lib.lib()
    prec = _lib.PREC_FP64 if precision == "fp64" else _lib.PREC_MIXED
    rng = np.random.default_rng(8)
    n, m, d = 20000, 128, 8
    x = rng.standard_normal((n, d))
    y = np.sin(x).sum(1) + 0.1 * rng.standard_normal(n)
    z = x[rng.choice(n, m, replace=False)]
    ls = np.exp(rng.uniform(-0.5, 0.5, d))
    dev = torch.device("cuda")
    th = torch.tensor(list(ls) + [1.2, 0.2, 0.1], dtype=torch.float64, device=dev)
    Z = torch.as_tensor(z, device=dev)

    def outputs():
        return (torch.zeros(1, dtype=torch.float64, device=dev),
                torch.zeros(d + 3, dtype=torch.float64, device=dev),
                torch.zeros((m, d), dtype=torch.float64, device=dev),
                torch.zeros(1, dtype=torch.int32, device=dev))

    X, Y = torch.as_tensor(x, device=dev), torch.as_tensor(y, device=dev)
    e, g, gz, info = outputs()
    ws = _lib.workspace(lib.gpk_collapsed_elbo_workspace_bytes(n, m, d, _lib.PREC_FP64), dev)
    _lib.call("gpk_collapsed_elbo", _lib.RBF, n, m, d, X.data_ptr(), d, Y.data_ptr(), Z.data_ptr(),
              d, th.data_ptr(), d, 1e-6, _lib.PREC_FP64, 1, e.data_ptr(), g.data_ptr(), gz.data_ptr(),
              info.data_ptr(), ws.data_ptr(), ws.numel(), _lib.stream_ptr(dev))
    torch.cuda.synchronize()
    ref = (float(e.item()), g.cpu().numpy(), gz.cpu().numpy())
    del ws

    barrier = threading.Barrier(2)
    slots, results, errors = {}, {}, []

    def rank_main(r):
        try:
            rows = shard_rows(n, 2, r)
            stream = torch.cuda.Stream(dev)
            with torch.cuda.stream(stream):
                Xr = torch.as_tensor(x[rows], device=dev)
                Yr = torch.as_tensor(y[rows], device=dev)
                er, gr, gzr, ir = outputs()
                nl = Xr.shape[0]
                wsr = _lib.workspace(lib.gpk_collapsed_elbo_workspace_bytes(nl, m, d, prec), dev)

                def hostsum(user, off, count, s):
                    view = wsr.narrow(0, int(off), int(count) * 8).view(torch.float64)
                    slots[r] = view.cpu().numpy()          # waits for this rank's stream
                    barrier.wait()
                    tot = slots[0] + slots[1]
                    barrier.wait()                          # both have read before the next exchange
                    view.copy_(torch.as_tensor(tot, device=dev))
                    return 0
                cb = _lib.ALLREDUCE_FN(hostsum)
                _lib.call("gpk_collapsed_elbo_sharded", _lib.RBF, nl, n, m, d, Xr.data_ptr(), d,
                          Yr.data_ptr(), Z.data_ptr(), d, th.data_ptr(), d, 1e-6, prec, 1,
                          er.data_ptr(), gr.data_ptr(), gzr.data_ptr(), ir.data_ptr(),
                          wsr.data_ptr(), wsr.numel(), stream.cuda_stream, cb, None)
                stream.synchronize()
                assert int(ir.item()) == 0
                results[r] = (float(er.item()), gr.cpu().numpy(), gzr.cpu().numpy())
        except Exception as exc:  # surfaced below
            errors.append(exc)
            barrier.abort()

    ts = [threading.Thread(target=rank_main, args=(r,)) for r in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=300)
    assert not errors, errors
    for r in range(2):
        val, gv, gzv = results[r]
        assert abs(val - ref[0]) <= vtol * abs(ref[0]), (r, val, ref[0])
        assert np.allclose(gv, ref[1], rtol=gtol, atol=gtol * np.abs(ref[1]).max())
        assert np.allclose(gzv, ref[2], rtol=gtol, atol=gtol * np.abs(ref[2]).max())
