"""Linear operators and the Cholesky / solve / logdet operations
(mirrors gpjax/linalg/operators.py, operations.py:22-222, utils.py:21-65).

Dense and Triangular operations run on the GPU through libgpk.so:
``lower_cholesky`` (operations.py:54-55) -> gpk_lower_cholesky,
``solve`` with a Triangular operator (operations.py:105-107) ->
gpk_solve_triangular, ``logdet`` (operations.py:142-144,163-165) ->
gpk_logdet_triangular of the Cholesky factor.  The reference solves and
log-determines Dense operators through LU factorisations; the matrices on the
GP path are symmetric positive definite, and here they are handled through
their Cholesky factor (identical values; a non-SPD Dense operator raises).
"""
from __future__ import annotations

import torch

from . import _lib


class LinearOperator:
    def to_dense(self) -> torch.Tensor:  # pragma: no cover - interface
        raise NotImplementedError

    @property
    def shape(self):
        return tuple(self.to_dense().shape)

    @property
    def dtype(self):
        return self.to_dense().dtype


class Dense(LinearOperator):
    def __init__(self, array: torch.Tensor):
        self.array = array

    def to_dense(self) -> torch.Tensor:
        return self.array

    @property
    def shape(self):
        return tuple(self.array.shape)


class Triangular(LinearOperator):
    def __init__(self, array: torch.Tensor, lower: bool = True):
        self.array = array
        self.lower = lower

    def to_dense(self) -> torch.Tensor:
        return self.array

    @property
    def shape(self):
        return tuple(self.array.shape)


class Diagonal(LinearOperator):
    def __init__(self, diagonal: torch.Tensor):
        self.diagonal = diagonal

    def to_dense(self) -> torch.Tensor:
        return torch.diag(self.diagonal)

    @property
    def shape(self):
        n = self.diagonal.shape[0]
        return (n, n)


class Identity(LinearOperator):
    def __init__(self, n: int, device=None):
        self.n = n
        self.device = device if device is not None else torch.device("cuda")

    def to_dense(self) -> torch.Tensor:
        return torch.eye(self.n, dtype=torch.float64, device=self.device)

    @property
    def shape(self):
        return (self.n, self.n)


def psd(A: LinearOperator) -> LinearOperator:
    """Tags an operator as positive semi-definite (utils.py:21-36)."""
    A.psd = True
    return A


def add_jitter(x: torch.Tensor, jitter: float = 1e-6) -> torch.Tensor:
    """x + I*jitter (utils.py:39-65)."""
    if x.ndim != 2 or x.shape[0] != x.shape[1]:
        raise ValueError("add_jitter expects a square matrix")
    out = x.clone()
    idx = torch.arange(x.shape[0], device=x.device)
    out[idx, idx] += jitter
    return out


def _dtype_code(t: torch.Tensor) -> int:
    if t.dtype == torch.float64:
        return _lib.F64
    if t.dtype == torch.float32:
        return _lib.F32
    raise TypeError(f"unsupported dtype {t.dtype}")


def cholesky_dense(A: torch.Tensor, check: bool = False) -> tuple[torch.Tensor, torch.Tensor]:
    """Lower Cholesky factor of A on the GPU; returns (L, info[1] int32 device)."""
    dev = _lib.require_cuda(A)
    L = A.detach().contiguous().clone()
    n = L.shape[0]
    info = torch.zeros(1, dtype=torch.int32, device=dev)
    _lib.call("gpk_lower_cholesky", n, _dtype_code(L), L.data_ptr(), L.stride(0), None,
              info.data_ptr(), _lib.stream_ptr(dev))
    if check and int(info.item()) != 0:
        raise ValueError(f"matrix is not positive definite (leading minor {int(info.item())})")
    return L, info


def lower_cholesky(A: LinearOperator) -> LinearOperator:
    """Lower Cholesky factor (operations.py:22-70)."""
    if isinstance(A, Identity):
        return A
    if isinstance(A, Diagonal):
        return Diagonal(torch.sqrt(A.diagonal))
    if isinstance(A, Triangular) and A.lower:
        return A
    L, _ = cholesky_dense(A.to_dense())
    return Triangular(L, lower=True)


def _solve(T: torch.Tensor, B: torch.Tensor, upper: bool, trans: bool) -> torch.Tensor:
    dev = _lib.require_cuda(T, B)
    T = T.detach().contiguous()
    squeeze = B.ndim == 1
    X = (B[:, None] if squeeze else B).detach().to(T.dtype).contiguous().clone()
    n, k = X.shape
    nbytes = _lib.lib().gpk_solve_triangular_ex_workspace_bytes(n, k, _dtype_code(T), int(upper))
    ws = _lib.workspace(nbytes, dev)
    _lib.call("gpk_solve_triangular_ex", n, k, _dtype_code(T), int(upper), int(trans),
              T.data_ptr(), T.stride(0), X.data_ptr(), X.stride(0), ws.data_ptr(), ws.numel(),
              _lib.stream_ptr(dev))
    return X[:, 0] if squeeze else X


def _solve_lower(L: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
    return _solve(L, B, upper=False, trans=False)


def solve_triangular(T: torch.Tensor, B: torch.Tensor, lower: bool = True,
                     trans: bool = False) -> torch.Tensor:
    """op(T) X = B for triangular T (jsp.linalg.solve_triangular with ``lower``
    and ``trans``), one library call."""
    return _solve(T, B, upper=not lower, trans=trans)


def matmul(A: torch.Tensor, B: torch.Tensor, transa: bool = False,
           transb: bool = False, alpha: float = 1.0) -> torch.Tensor:
    """alpha op(A) op(B) in float64 through the library's GEMM (gpk_gemm_f64)."""
    dev = _lib.require_cuda(A, B)
    A = A.detach().to(torch.float64).contiguous()
    B = B.detach().to(torch.float64).contiguous()
    M, K = (A.shape[1], A.shape[0]) if transa else (A.shape[0], A.shape[1])
    KB, N = (B.shape[1], B.shape[0]) if transb else (B.shape[0], B.shape[1])
    if K != KB:
        raise ValueError(f"inner dimensions differ: {K} and {KB}")
    C = torch.empty((M, N), dtype=torch.float64, device=dev)
    nbytes = _lib.lib().gpk_gemm_f64_workspace_bytes(int(transa), int(transb), M, N, K)
    ws = _lib.workspace(nbytes, dev)
    _lib.call("gpk_gemm_f64", int(transa), int(transb), M, N, K, float(alpha), A.data_ptr(),
              A.stride(0), B.data_ptr(), B.stride(0), 0.0, C.data_ptr(), N, ws.data_ptr(),
              ws.numel(), _lib.stream_ptr(dev))
    return C


def solve(A: LinearOperator, b: torch.Tensor) -> torch.Tensor:
    """Solves A x = b (operations.py:73-120)."""
    squeeze = b.ndim == 1
    B = b[:, None] if squeeze else b
    if isinstance(A, Identity):
        res = B
    elif isinstance(A, Diagonal):
        res = B / A.diagonal[:, None]
    elif isinstance(A, Triangular):
        res = solve_triangular(A.array, B, lower=A.lower)
    else:
        L, _ = cholesky_dense(A.to_dense(), check=True)
        res = solve_triangular(L, _solve_lower(L, B), trans=True)  # L^T x = L^-1 b
    return res[:, 0] if squeeze else res


def logdet(A: LinearOperator) -> torch.Tensor:
    """log|A| (operations.py:123-181)."""
    if isinstance(A, Identity):
        return torch.zeros((), dtype=torch.float64)
    if isinstance(A, Diagonal):
        return torch.sum(torch.log(A.diagonal))
    if isinstance(A, Triangular):
        T = A.array.detach().contiguous()
        dev = _lib.require_cuda(T)
        out = torch.empty(1, dtype=torch.float64, device=dev)
        _lib.call("gpk_logdet_triangular", T.shape[0], _dtype_code(T), T.data_ptr(), T.stride(0),
                  out.data_ptr(), _lib.stream_ptr(dev))
        return out[0]
    L, _ = cholesky_dense(A.to_dense(), check=True)
    return 2.0 * logdet(Triangular(L))


def diag(A: LinearOperator) -> torch.Tensor:
    """Diagonal of an operator (operations.py:184-222)."""
    if isinstance(A, Diagonal):
        return A.diagonal
    if isinstance(A, Identity):
        return torch.ones(A.n, dtype=torch.float64, device=A.device)
    return torch.diagonal(A.to_dense())
