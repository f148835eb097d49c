"""Library-wide settings.

``default_precision`` selects the arithmetic of the objectives and predict:
"fp64" computes every step in float64 (the reference's precision under
jax_enable_x64); "mixed" uses the float32 Gram with a tensor-core
factorisation and adjoint (split-TF32, and split-float16 on row-scaled
operands for the large products) and float64 refinement.
"""
from __future__ import annotations

from . import _lib

_PRECISIONS = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}
default_precision = "fp64"


def precision_code(precision: str | None) -> int:
    p = default_precision if precision is None else precision
    if p not in _PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}, got {p!r}")
    return _PRECISIONS[p]


def set_precision(precision: str) -> None:
    global default_precision
    precision_code(precision)
    default_precision = precision
