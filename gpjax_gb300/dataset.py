"""Dataset container (mirrors gpjax/dataset.py:26-126)."""
from __future__ import annotations

import warnings

import numpy as np
import torch


class Dataset:
    """Inputs X [n, d] and outputs y [n, q] as float64 CUDA tensors.

    As the reference's Dataset (gpjax/dataset.py:26-126): row counts must
    agree, non-float64 inputs are converted with a warning, ``+`` stacks two
    datasets (a side missing from either is None in the sum), and
    ``is_supervised`` / ``is_unsupervised`` tell X-and-y from y-only data.
    One extension: a 1-D X or y is taken as a single column.
    """

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

    def is_supervised(self) -> bool:
        return self.X is not None and self.y is not None

    def is_unsupervised(self) -> bool:
        return self.X is None and self.y is not None

    @property
    def n(self) -> int:
        if self.X is not None:
            return int(self.X.shape[0])
        return 0 if self.y is None else int(self.y.shape[0])

    @property
    def in_dim(self) -> int:
        return int(self.X.shape[1])

    def __add__(self, other: "Dataset") -> "Dataset":
        X = torch.cat([self.X, other.X]) if self.X is not None and other.X is not None else None
        y = torch.cat([self.y, other.y]) if self.y is not None and other.y is not None else None
        dev = (X if X is not None else y).device if (X is not None or y is not None) else None
        return Dataset(X=X, y=y, device=dev)

    def __repr__(self) -> str:
        dim = self.in_dim if self.X is not None else 0
        return f"Dataset(Number of observations: {self.n} - Input dimension: {dim})"


def _to(a, dev) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=torch.float64)
    return torch.as_tensor(np.asarray(a, dtype=np.float64), device=dev)
