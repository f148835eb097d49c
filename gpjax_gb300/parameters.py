"""Parameter containers (mirrors gpjax/parameters.py:69-103).

A parameter holds its value as a float64 torch tensor in ``.value``.  Values
are the reference's constrained coordinates (lengthscale > 0, variance >= 0,
obs_stddev >= 0); gradients from the objectives land in ``.value.grad`` when
the tensor requires grad, the counterpart of ``jax.grad`` over an
``nnx.State`` in the reference (tests/test_objectives.py:68-85).
"""
from __future__ import annotations

import numpy as np
import torch


def _as_tensor(value, device=None) -> torch.Tensor:
    if isinstance(value, Parameter):
        return value.value
    if isinstance(value, torch.Tensor):
        t = value
        if t.dtype != torch.float64:
            t = t.to(torch.float64)
        return t if device is None else t.to(device)
    return torch.as_tensor(np.asarray(value, dtype=np.float64), device=device)


class Parameter:
    """A trainable value (gpjax.parameters.Parameter)."""

    _tag = "parameter"

    def __init__(self, value, tag: str | None = None, device=None):
        self.value = _as_tensor(value, device)
        if tag is not None:
            self._tag = tag
        self._check()

    def _check(self) -> None:
        pass

    @property
    def tag(self) -> str:
        return self._tag

    def requires_grad_(self, flag: bool = True) -> "Parameter":
        self.value = self.value.detach().requires_grad_(flag)
        return self

    def to(self, device) -> "Parameter":
        self.value = self.value.detach().to(device).requires_grad_(self.value.requires_grad)
        return self

    def __repr__(self) -> str:
        return f"{type(self).__name__}({self.value!r})"


class PositiveReal(Parameter):
    """Strictly positive parameter (parameters.py:83-88)."""

    _tag = "positive"

    def _check(self) -> None:
        v = self.value.detach()
        if v.numel() and not bool(torch.all(v > 0)):
            raise ValueError("PositiveReal requires values > 0")


class NonNegativeReal(Parameter):
    """Non-negative parameter (parameters.py:90-95)."""

    _tag = "non_negative"

    def _check(self) -> None:
        v = self.value.detach()
        if v.numel() and not bool(torch.all(v >= 0)):
            raise ValueError("NonNegativeReal requires values >= 0")


class Real(Parameter):
    """Unconstrained parameter (parameters.py:97-103)."""

    _tag = "real"


def softplus_inverse(x: torch.Tensor) -> torch.Tensor:
    """Inverse of the default softplus bijection (parameters.py:140-146)."""
    return x + torch.log(-torch.expm1(-x))
