"""Dataset container (mirrors gpjax/dataset.py:26-126)."""
from __future__ import annotations

import warnings

import numpy as np
import torch


class Dataset:
    """Inputs X [n, d] and outputs y [n, q] as float64 CUDA tensors."""

    def __init__(self, X=None, y=None, device=None):
        dev = device if device is not None else (
            torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu"))
        self.X = None if X is None else _to(X, dev)
        self.y = None if y is None else _to(y, dev)
        if self.X is not None and self.X.ndim == 1:
            self.X = self.X[:, None]
        if self.y is not None and self.y.ndim == 1:
            self.y = self.y[:, None]
        if self.X is not None and self.y is not None and self.X.shape[0] != self.y.shape[0]:
            raise ValueError(
                f"Inputs, X, and outputs, y, must have the same number of rows. "
                f"Got X.shape={tuple(self.X.shape)} and y.shape={tuple(self.y.shape)}.")
        for name, arr in (("X", X), ("y", y)):
            if arr is not None and getattr(arr, "dtype", None) not in (np.float64, torch.float64):
                warnings.warn(f"{name} is not of type float64; converted to float64", UserWarning)

    @property
    def n(self) -> int:
        return 0 if self.X is None else int(self.X.shape[0])

    @property
    def in_dim(self) -> int:
        return int(self.X.shape[1])

    def __add__(self, other: "Dataset") -> "Dataset":
        return Dataset(torch.cat([self.X, other.X]), torch.cat([self.y, other.y]))

    def __repr__(self) -> str:
        return f"Dataset(n={self.n}, X={tuple(self.X.shape)}, y={tuple(self.y.shape)})"


def _to(a, dev) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=torch.float64)
    return torch.as_tensor(np.asarray(a, dtype=np.float64), device=dev)
