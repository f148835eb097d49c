"""Training loops over the GPU objectives (mirrors gpjax/fit.py:44-361).

``fit_scipy`` and ``fit_lbfgs`` optimise the trainable parameters of a model
in the reference's unconstrained coordinates: positive and non-negative
parameters through the softplus bijection, real ones unchanged
(parameters.py:140-146, ``DEFAULT_BIJECTION``).  Each evaluation is one
library call returning the objective with its constrained gradient; torch's
autograd applies the bijection's chain rule (d/du = d/dtheta * sigmoid(u)).
The evaluations of one fit share a resident device workspace
(``_lib.resident_workspace``), so the n^2 buffers of the factorisation are
allocated once per fit, not once per line-search step.
"""
from __future__ import annotations

import contextlib

import numpy as np
import torch

from . import _lib
from .objectives import named_parameters
from .parameters import Parameter


def _bijection(tag: str):
    """(to constrained, to unconstrained) for a parameter tag (parameters.py:140-146)."""
    if tag in ("positive", "non_negative"):
        return (torch.nn.functional.softplus,
                lambda v: v + torch.log(-torch.expm1(-v)))  # softplus inverse
    if tag == "real":
        return (lambda u: u, lambda v: v)
    raise ValueError(f"no bijection for parameter tag {tag!r}")


class _Unconstrained:
    """The model's trainable parameters as one flat unconstrained float64 vector."""

    def __init__(self, model, device):
        self.params: dict[str, Parameter] = named_parameters(model)
        if not self.params:
            raise ValueError("the model has no trainable parameters")
        self.device = device
        self.shapes = [p.value.shape for p in self.params.values()]
        self.sizes = [int(p.value.numel()) for p in self.params.values()]
        self.maps = [_bijection(p.tag) for p in self.params.values()]

    def flat(self) -> np.ndarray:
        parts = [inv(p.value.detach().to(self.device)).reshape(-1)
                 for p, (_, inv) in zip(self.params.values(), self.maps)]
        return torch.cat(parts).cpu().numpy().astype(np.float64)

    def assign(self, u: torch.Tensor) -> None:
        """Sets every parameter to the constrained image of its slice of u (keeps the graph)."""
        off = 0
        for p, shape, size, (fwd, _) in zip(self.params.values(), self.shapes, self.sizes,
                                            self.maps):
            p.value = fwd(u[off:off + size]).reshape(shape)
            off += size

    def value_and_grad(self, objective, model, data, x: np.ndarray):
        u = torch.as_tensor(x, dtype=torch.float64, device=self.device).requires_grad_(True)
        self.assign(u)
        val = objective(model, data)
        (g,) = torch.autograd.grad(val, u)
        return float(val.detach()), g.detach().cpu().numpy().astype(np.float64)

    def finish(self, x: np.ndarray) -> None:
        with torch.no_grad():
            self.assign(torch.as_tensor(x, dtype=torch.float64, device=self.device))
        for p in self.params.values():
            p.value = p.value.detach()


def _device_of(data):
    return data.X.device if isinstance(data.X, torch.Tensor) else \
        torch.device("cuda", torch.cuda.current_device())


def _resident(dev):
    return _lib.resident_workspace(dev) if dev.type == "cuda" else contextlib.nullcontext()


def _check(model, objective, train_data, max_iters):
    if not callable(objective):
        raise TypeError("objective must be callable: objective(model, data) -> scalar")
    if not hasattr(train_data, "X") or not hasattr(train_data, "y"):
        raise TypeError("train_data must be a Dataset")
    if not isinstance(max_iters, int) or max_iters <= 0:
        raise ValueError("max_iters must be a positive integer")


def fit_scipy(*, model, objective, train_data, max_iters: int = 500, verbose: bool = True,
              safe: bool = True):
    """Minimise ``objective(model, train_data)`` with scipy's BFGS over the
    unconstrained parameters (fit.py:183-256).  Returns (model, history) with
    the loss at the start and after every iteration."""
    from scipy.optimize import minimize

    if safe:
        _check(model, objective, train_data, max_iters)
    dev = _device_of(train_data)
    state = _Unconstrained(model, dev)
    x0 = state.flat()
    with _resident(dev):
        fun = lambda x: state.value_and_grad(objective, model, train_data, x)  # noqa: E731
        history = [fun(x0)[0]]
        res = minimize(fun=fun, x0=x0, jac=True,
                       callback=lambda x: history.append(fun(x)[0]),
                       options={"maxiter": max_iters, "disp": verbose})
    state.finish(res.x)
    return model, np.asarray(history)


def fit_lbfgs(*, model, objective, train_data, max_iters: int = 100, safe: bool = True,
              max_linesearch_steps: int = 32, gtol: float = 1e-5):
    """Minimise ``objective(model, train_data)`` with limited-memory BFGS over
    the unconstrained parameters (fit.py:259-361; scipy's L-BFGS-B with its
    line search standing in for optax's zoom line search).  Stops after
    max_iters iterations or when the gradient's largest component falls below
    gtol.  Returns (model, final loss)."""
    from scipy.optimize import minimize

    if safe:
        _check(model, objective, train_data, max_iters)
    dev = _device_of(train_data)
    state = _Unconstrained(model, dev)
    with _resident(dev):
        res = minimize(fun=lambda x: state.value_and_grad(objective, model, train_data, x),
                       x0=state.flat(), jac=True, method="L-BFGS-B",
                       options={"maxiter": max_iters, "maxls": max_linesearch_steps,
                                "gtol": gtol})
    state.finish(res.x)
    return model, float(res.fun)


def fit(*, model, objective, train_data, num_iters: int = 100, learning_rate: float = 0.01,
        verbose: bool = False, safe: bool = True):
    """First-order loop (fit.py:44-180 with ``optax.adam``): Adam steps on the
    unconstrained parameters over the full dataset.  Returns (model, history)."""
    if safe:
        _check(model, objective, train_data, num_iters)
    dev = _device_of(train_data)
    state = _Unconstrained(model, dev)
    u = torch.as_tensor(state.flat(), dtype=torch.float64, device=dev).requires_grad_(True)
    opt = torch.optim.Adam([u], lr=learning_rate)
    history = []
    with _resident(dev):
        for it in range(num_iters):
            opt.zero_grad()
            state.assign(u)
            loss = objective(model, train_data)
            loss.backward()
            opt.step()
            history.append(float(loss.detach()))
            if verbose and it % 10 == 0:
                print(f"iter {it}: {history[-1]:.6f}")
    state.finish(u.detach().cpu().numpy())
    return model, np.asarray(history)
