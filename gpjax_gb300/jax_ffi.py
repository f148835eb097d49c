"""JAX entry points: the library's objectives as XLA FFI custom calls.

A GPJax user keeps the reference's API and swaps the objective:

    import gpjax_gb300.jax_ffi as gfx
    gfx.register()                      # once per process
    loss = lambda p, d: -gfx.conjugate_mll(p, d)       # objectives.py:36-107
    gpx.fit_scipy(model=posterior, objective=loss, train_data=D)

``conjugate_mll`` and ``collapsed_elbo`` read the constrained parameter values
of the GPJax posterior / variational family (``kernel.lengthscale.value``,
``kernel.variance.value``, ``likelihood.obs_stddev.value``, the constant mean),
pack them into the C ABI's theta vector with jnp operations, and call the
custom call under ``jax.custom_vjp``: the forward pass returns the value and
keeps the gradient the library computed with it, the backward pass scales that
gradient by the cotangent (the counterpart of ``jax.value_and_grad`` at
``fit.py:160,233``).  Gradients then flow back through the packing to the
``nnx`` parameters.

The handlers live in ``ffi/gpk_ffi.cc`` (XLA_FFI_DEFINE_HANDLER_SYMBOL over
``include/gpk.h``); :func:`build` compiles them against jaxlib's headers
(``jax.ffi.include_dir()``) and ``libgpk.so``.  Without jax this module
imports, :func:`available` is False, and every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
from functools import partial

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ffi", "gpk_ffi.cc")
LIB = os.path.join(HERE, "libgpk_ffi.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

# kernel codes of include/gpk.h by the reference's kernel class names
KINDS = {"RBF": 0, "Matern32": 1, "Matern52": 2, "Matern12": 3, "RationalQuadratic": 4}
PRECISIONS = {"fp64": 0, "mixed": 1}
TARGETS = {"gpk_conjugate_mll": "GpkConjugateMll", "gpk_collapsed_elbo": "GpkCollapsedElbo",
           "gpk_predict": "GpkPredict"}

try:  # jax is optional: only the JAX entry points need it
    import jax
    import jax.numpy as jnp
    _HAVE_JAX = hasattr(jax, "ffi")
except ImportError:  # pragma: no cover - depends on the environment
    jax = jnp = None
    _HAVE_JAX = False

_registered = False


def available() -> bool:
    """True when jax (with jax.ffi) is importable."""
    return _HAVE_JAX


def _require():
    if not _HAVE_JAX:
        raise RuntimeError("gpjax_gb300.jax_ffi needs jax with jax.ffi (jax >= 0.4.31); "
                           "use gpjax_gb300.objectives for torch callers")


def build(force: bool = False) -> str:
    """Compiles ffi/gpk_ffi.cc against jaxlib's FFI headers and libgpk.so."""
    _require()
    from . import _build
    gpk = _build.build()
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("a C++17 compiler is needed to build the FFI handlers")
    cuda_inc = "/usr/local/cuda/include"
    cmd = [cxx, "-O2", "-std=c++17", "-shared", "-fPIC", SRC, "-o", LIB,
           f"-I{jax.ffi.include_dir()}", f"-I{INCLUDE}", f"-I{cuda_inc}", gpk,
           f"-Wl,-rpath,{HERE}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the FFI handlers failed:\n{r.stderr}")
    return LIB


def register() -> None:
    """Registers the three custom-call targets for the CUDA platform (once)."""
    global _registered
    _require()
    if _registered:
        return
    lib = ctypes.cdll.LoadLibrary(build())
    for name, sym in TARGETS.items():
        jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(getattr(lib, sym)), platform="CUDA")
    _registered = True


def _kernel_code(kernel) -> int:
    name = type(kernel).__name__
    if name not in KINDS:
        raise NotImplementedError(f"no GPU kernel for {name}; supported: {sorted(KINDS)}")
    return KINDS[name]


def _value(v):
    return v.value if hasattr(v, "value") else v


def pack_theta(kernel, obs_stddev, constant):
    """[lengthscale..., variance, obs_stddev, constant (, alpha)] in float64,
    the theta layout of include/gpk.h; returns (theta, n_ls)."""
    ls = jnp.atleast_1d(jnp.asarray(_value(kernel.lengthscale), jnp.float64))
    parts = [ls, jnp.reshape(jnp.asarray(_value(kernel.variance), jnp.float64), (1,)),
             jnp.reshape(jnp.asarray(obs_stddev, jnp.float64), (1,)),
             jnp.reshape(jnp.asarray(constant, jnp.float64), (1,))]
    if _kernel_code(kernel) == KINDS["RationalQuadratic"]:
        parts.append(jnp.reshape(jnp.asarray(_value(kernel.alpha), jnp.float64), (1,)))
    return jnp.concatenate(parts), int(ls.shape[0])


def _mean_constant(mean_function):
    c = getattr(mean_function, "constant", None)
    return 0.0 if c is None else jnp.reshape(jnp.asarray(_value(c), jnp.float64), ())


def _mll_call(theta, x, y, kind, n_ls, jitter, precision, want_grad):
    out = (jax.ShapeDtypeStruct((), jnp.float64), jax.ShapeDtypeStruct(theta.shape, jnp.float64),
           jax.ShapeDtypeStruct((), jnp.int32))
    return jax.ffi.ffi_call("gpk_conjugate_mll", out)(
        x, y, theta, kind=np.int32(kind), n_ls=np.int32(n_ls), jitter=np.float64(jitter),
        precision=np.int32(precision), want_grad=np.int32(want_grad))


if _HAVE_JAX:
    @partial(jax.custom_vjp, nondiff_argnums=(3, 4, 5, 6))
    def _mll(theta, x, y, kind, n_ls, jitter, precision):
        return _mll_call(theta, x, y, kind, n_ls, jitter, precision, 0)[0]

    def _mll_fwd(theta, x, y, kind, n_ls, jitter, precision):
        val, grad, _ = _mll_call(theta, x, y, kind, n_ls, jitter, precision, 1)
        return val, (grad, x, y)

    def _mll_bwd(kind, n_ls, jitter, precision, res, g):
        grad, x, y = res
        return g * grad, jnp.zeros_like(x), jnp.zeros_like(y)

    _mll.defvjp(_mll_fwd, _mll_bwd)

    def _elbo_call(theta, z, x, y, kind, n_ls, jitter, precision, want_grad):
        out = (jax.ShapeDtypeStruct((), jnp.float64),
               jax.ShapeDtypeStruct(theta.shape, jnp.float64),
               jax.ShapeDtypeStruct(z.shape, jnp.float64), jax.ShapeDtypeStruct((), jnp.int32))
        return jax.ffi.ffi_call("gpk_collapsed_elbo", out)(
            x, y, z, theta, kind=np.int32(kind), n_ls=np.int32(n_ls), jitter=np.float64(jitter),
            precision=np.int32(precision), want_grad=np.int32(want_grad))

    @partial(jax.custom_vjp, nondiff_argnums=(4, 5, 6, 7))
    def _elbo(theta, z, x, y, kind, n_ls, jitter, precision):
        return _elbo_call(theta, z, x, y, kind, n_ls, jitter, precision, 0)[0]

    def _elbo_fwd(theta, z, x, y, kind, n_ls, jitter, precision):
        val, grad, gz, _ = _elbo_call(theta, z, x, y, kind, n_ls, jitter, precision, 1)
        return val, (grad, gz, x, y)

    def _elbo_bwd(kind, n_ls, jitter, precision, res, g):
        grad, gz, x, y = res
        return g * grad, g * gz, jnp.zeros_like(x), jnp.zeros_like(y)

    _elbo.defvjp(_elbo_fwd, _elbo_bwd)


def conjugate_mll(posterior, data, precision: str = "fp64"):
    """Drop-in for gpjax.objectives.conjugate_mll (objectives.py:36-107) on the GPU."""
    _require()
    register()
    prior = posterior.prior
    kernel = prior.kernel
    theta, n_ls = pack_theta(kernel, _value(posterior.likelihood.obs_stddev),
                             _mean_constant(prior.mean_function))
    x = jnp.asarray(data.X, jnp.float64)
    y = jnp.reshape(jnp.asarray(data.y, jnp.float64), (-1,))
    return _mll(theta, x, y, _kernel_code(kernel), n_ls, float(prior.jitter),
                PRECISIONS[precision])


def collapsed_elbo(variational_family, data, precision: str = "fp64"):
    """Drop-in for gpjax.objectives.collapsed_elbo (objectives.py:321-416) on the GPU."""
    _require()
    register()
    post = variational_family.posterior
    kernel = post.prior.kernel
    theta, n_ls = pack_theta(kernel, _value(post.likelihood.obs_stddev),
                             _mean_constant(post.prior.mean_function))
    z = jnp.asarray(_value(variational_family.inducing_inputs), jnp.float64)
    x = jnp.asarray(data.X, jnp.float64)
    y = jnp.reshape(jnp.asarray(data.y, jnp.float64), (-1,))
    return _elbo(theta, z, x, y, _kernel_code(kernel), n_ls,
                 float(variational_family.jitter), PRECISIONS[precision])


def predict_mean_variance(posterior, test_inputs, train_data, precision: str = "fp64"):
    """Predictive mean and variance of ConjugatePosterior.predict (gps.py:443-526)."""
    _require()
    register()
    prior = posterior.prior
    kernel = prior.kernel
    theta, n_ls = pack_theta(kernel, _value(posterior.likelihood.obs_stddev),
                             _mean_constant(prior.mean_function))
    x = jnp.asarray(train_data.X, jnp.float64)
    y = jnp.reshape(jnp.asarray(train_data.y, jnp.float64), (-1,))
    xt = jnp.asarray(test_inputs, jnp.float64)
    t = xt.shape[0]
    out = (jax.ShapeDtypeStruct((t,), jnp.float64), jax.ShapeDtypeStruct((t,), jnp.float64),
           jax.ShapeDtypeStruct((), jnp.int32))
    mean, var, _ = jax.ffi.ffi_call("gpk_predict", out)(
        x, y, xt, theta, kind=np.int32(_kernel_code(kernel)), n_ls=np.int32(n_ls),
        jitter=np.float64(posterior.jitter), prior_jitter=np.float64(prior.jitter),
        precision=np.int32(PRECISIONS[precision]))
    return mean, var
