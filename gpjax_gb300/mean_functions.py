"""Mean functions (mirrors gpjax/mean_functions.py:131-165)."""
from __future__ import annotations

import torch

from .parameters import Parameter


class Constant:
    """m(x) = c.  A Parameter constant is trainable; a plain value is fixed."""

    def __init__(self, constant=0.0):
        self.constant = constant if isinstance(constant, Parameter) else torch.as_tensor(
            float(constant), dtype=torch.float64)

    def value_tensor(self, device) -> torch.Tensor:
        c = self.constant.value if isinstance(self.constant, Parameter) else self.constant
        return c.reshape(()).to(device)

    def __call__(self, x: torch.Tensor) -> torch.Tensor:
        return torch.ones((x.shape[0], 1), dtype=torch.float64, device=x.device) * \
            self.value_tensor(x.device)


class Zero(Constant):
    """m(x) = 0, not trainable."""

    def __init__(self):
        super().__init__(constant=0.0)
