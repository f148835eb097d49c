"""ctypes binding of the C ABI declared in include/gpk.h.

The shared library is loaded from the package directory.  There is no
fallback: every computation in this package runs through libgpk.so on a CUDA
device, and a missing library or device raises immediately.
"""
from __future__ import annotations

import ctypes
import os

import torch

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libgpk.so")

# enums (include/gpk.h)
RBF, MATERN32, MATERN52, MATERN12, RATIONAL_QUADRATIC = 0, 1, 2, 3, 4
F64, F32 = 0, 1
PREC_FP64, PREC_MIXED = 0, 1

_c_i64 = ctypes.c_int64
_c_int = ctypes.c_int
_c_dbl = ctypes.c_double
_c_ptr = ctypes.c_void_p
_c_size = ctypes.c_size_t

# name -> (restype, argtypes)
SIGNATURES = {
    "gpk_version": (_c_int, []),
    "gpk_status_string": (ctypes.c_char_p, [_c_int]),
    "gpk_launch_count": (ctypes.c_longlong, []),
    "gpk_set_profile_events": (None, [ctypes.POINTER(ctypes.c_void_p), _c_int]),
    "gpk_cross_covariance": (_c_int, [_c_int, _c_i64, _c_i64, _c_int, _c_ptr, _c_i64, _c_ptr,
                                      _c_i64, _c_ptr, _c_int, _c_int, _c_ptr, _c_i64, _c_ptr]),
    "gpk_gram": (_c_int, [_c_int, _c_i64, _c_int, _c_ptr, _c_i64, _c_ptr, _c_int, _c_int, _c_ptr,
                          _c_i64, _c_ptr]),
    "gpk_cross_covariance_vjp_workspace_bytes": (_c_size, [_c_i64, _c_i64, _c_int]),
    "gpk_cross_covariance_vjp": (_c_int, [_c_int, _c_i64, _c_i64, _c_int, _c_ptr, _c_i64, _c_ptr,
                                          _c_i64, _c_ptr, _c_int, _c_ptr, _c_i64, _c_ptr, _c_ptr,
                                          _c_ptr, _c_ptr, _c_size, _c_ptr]),
    "gpk_diagonal": (_c_int, [_c_int, _c_i64, _c_int, _c_ptr, _c_i64, _c_ptr, _c_int, _c_ptr,
                              _c_ptr]),
    "gpk_lower_cholesky": (_c_int, [_c_i64, _c_int, _c_ptr, _c_i64, _c_ptr, _c_ptr, _c_ptr]),
    "gpk_solve_triangular_workspace_bytes": (_c_size, [_c_i64, _c_i64, _c_int]),
    "gpk_solve_triangular": (_c_int, [_c_i64, _c_i64, _c_int, _c_ptr, _c_i64, _c_ptr, _c_i64,
                                      _c_ptr, _c_size, _c_ptr]),
    "gpk_solve_triangular_ex_workspace_bytes": (_c_size, [_c_i64, _c_i64, _c_int, _c_int]),
    "gpk_solve_triangular_ex": (_c_int, [_c_i64, _c_i64, _c_int, _c_int, _c_int, _c_ptr, _c_i64,
                                         _c_ptr, _c_i64, _c_ptr, _c_size, _c_ptr]),
    "gpk_gemm_f64_workspace_bytes": (_c_size, [_c_int, _c_int, _c_i64, _c_i64, _c_i64]),
    "gpk_gemm_f64": (_c_int, [_c_int, _c_int, _c_i64, _c_i64, _c_i64, _c_dbl, _c_ptr, _c_i64,
                              _c_ptr, _c_i64, _c_dbl, _c_ptr, _c_i64, _c_ptr, _c_size, _c_ptr]),
    "gpk_logdet_triangular": (_c_int, [_c_i64, _c_int, _c_ptr, _c_i64, _c_ptr, _c_ptr]),
    "gpk_conjugate_mll_workspace_bytes": (_c_size, [_c_i64, _c_int, _c_int]),
    "gpk_conjugate_mll": (_c_int, [_c_int, _c_i64, _c_int, _c_ptr, _c_i64, _c_ptr, _c_ptr, _c_int,
                                   _c_dbl, _c_int, _c_int, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_size,
                                   _c_ptr]),
    "gpk_conjugate_mll_batched_workspace_bytes": (_c_size, [_c_int, _c_ptr, _c_ptr]),
    "gpk_conjugate_mll_batched": (_c_int, [_c_int, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr,
                                           _c_ptr, _c_ptr, _c_dbl, _c_int, _c_ptr, _c_ptr,
                                           _c_ptr, _c_ptr, _c_size, _c_ptr]),
    "gpk_batch_plan_create": (_c_int, [_c_int, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr,
                                       _c_ptr, _c_ptr, _c_dbl, _c_int, _c_ptr, _c_ptr, _c_ptr,
                                       _c_int, _c_ptr]),
    "gpk_batch_plan_workspace_bytes": (_c_size, [_c_ptr]),
    "gpk_batch_plan_config": (_c_int, [_c_ptr, _c_i64]),
    "gpk_batch_plan_config_count": (_c_int, []),
    "gpk_batch_plan_force_config": (_c_int, [_c_ptr, _c_int]),
    "gpk_batch_plan_selftest_stall": (_c_int, [_c_ptr, ctypes.c_longlong]),
    "gpk_batch_plan_execute": (_c_int, [_c_ptr, _c_ptr, _c_size, _c_ptr]),
    "gpk_batch_plan_destroy": (_c_int, [_c_ptr]),
    "gpk_conjugate_loocv_workspace_bytes": (_c_size, [_c_i64, _c_int]),
    "gpk_conjugate_loocv": (_c_int, [_c_int, _c_i64, _c_int, _c_ptr, _c_i64, _c_ptr, _c_ptr,
                                     _c_int, _c_dbl, _c_int, _c_ptr, _c_ptr, _c_ptr, _c_ptr,
                                     _c_size, _c_ptr]),
    "gpk_conjugate_mll_noalloc_max_n": (_c_size, []),
    "gpk_conjugate_mll_noalloc": (_c_int, [_c_int, _c_i64, _c_int, _c_ptr, _c_i64, _c_ptr, _c_ptr,
                                           _c_int, _c_dbl, _c_int, _c_ptr, _c_ptr, _c_ptr,
                                           _c_ptr]),
    "gpk_collapsed_elbo_workspace_bytes": (_c_size, [_c_i64, _c_i64, _c_int, _c_int]),
    "gpk_collapsed_elbo": (_c_int, [_c_int, _c_i64, _c_i64, _c_int, _c_ptr, _c_i64, _c_ptr,
                                    _c_ptr, _c_i64, _c_ptr, _c_int, _c_dbl, _c_int, _c_int,
                                    _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_ptr, _c_size, _c_ptr]),
    "gpk_collapsed_elbo_sharded": (_c_int, [_c_int, _c_i64, _c_i64, _c_i64, _c_int, _c_ptr, _c_i64,
                                            _c_ptr, _c_ptr, _c_i64, _c_ptr, _c_int, _c_dbl,
                                            _c_int, _c_int, _c_ptr, _c_ptr, _c_ptr, _c_ptr,
                                            _c_ptr, _c_size, _c_ptr, _c_ptr, _c_ptr]),
    "gpk_gemm_tf32x3_workspace_bytes": (_c_size, [_c_i64, _c_i64, _c_i64]),
    "gpk_gemm_tf32x3": (_c_int, [_c_i64, _c_i64, _c_i64, ctypes.c_float, _c_ptr, _c_i64, _c_ptr,
                                 _c_i64, ctypes.c_float, _c_ptr, _c_i64, _c_int, _c_ptr, _c_ptr,
                                 _c_size, _c_ptr]),
    "gpk_selftest_wait_timeout_workspace_bytes": (_c_size, []),
    "gpk_selftest_wait_timeout": (_c_int, [_c_ptr, _c_ptr, _c_size, _c_ptr]),
    "gpk_predict_workspace_bytes": (_c_size, [_c_i64, _c_i64, _c_int, _c_int]),
    "gpk_predict": (_c_int, [_c_int, _c_i64, _c_i64, _c_int, _c_ptr, _c_i64, _c_ptr, _c_ptr,
                             _c_i64, _c_ptr, _c_int, _c_dbl, _c_dbl, _c_int, _c_ptr, _c_ptr,
                             _c_ptr, _c_i64, _c_ptr, _c_ptr, _c_size, _c_ptr]),
}

# int (*gpk_allreduce_fn)(void* user, size_t byte_offset, int64_t count, cudaStream_t)
ALLREDUCE_FN = ctypes.CFUNCTYPE(_c_int, _c_ptr, _c_size, _c_i64, _c_ptr)

_LIB = None


class GPKError(RuntimeError):
    """A non-zero gpk_status from the C ABI."""

    def __init__(self, fn: str, status: int):
        msg = lib().gpk_status_string(status).decode()
        super().__init__(f"{fn} failed: {msg} (status {status})")
        self.status = status


def lib() -> ctypes.CDLL:
    """Loads libgpk.so once and declares every exported signature."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing; build it with `python -m gpjax_gb300._build` "
                "(nvcc, sm_103a).  There is no CPU fallback.")
        handle = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name, None)
            if fn is None:
                continue  # call() raises for an entry point this build lacks
            fn.restype = res
            fn.argtypes = args
        _LIB = handle
    return _LIB


def call(name: str, *args) -> None:
    """Calls a gpk_* entry point and raises GPKError on a non-zero status."""
    fn = getattr(lib(), name, None)
    if fn is None:
        raise RuntimeError(f"{name} is not exported by {LIB_PATH}")
    st = fn(*args)
    if st != 0:
        raise GPKError(name, st)


def require_cuda(*tensors: torch.Tensor) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("gpjax_gb300 needs a CUDA device (GB300, sm_103a); none is visible")
    for t in tensors:
        if t is not None and not t.is_cuda:
            raise ValueError("expected CUDA tensors")
    return tensors[0].device if tensors else torch.device("cuda")


def stream_ptr(device: torch.device | None = None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


_RESIDENT: dict = {}  # device index -> uint8 buffer, while a resident_workspace() is open


def workspace(nbytes: int, device: torch.device) -> torch.Tensor:
    """Caller-owned workspace for one call (the library never allocates).  Inside
    ``resident_workspace(device)`` every call gets the front of one buffer that
    stays allocated between calls (grown when a call needs more)."""
    nbytes = max(int(nbytes), 256)
    idx = torch.device(device).index
    if idx is None:
        idx = torch.cuda.current_device()
    if idx in _RESIDENT:
        buf = _RESIDENT[idx]
        if buf is None or buf.numel() < nbytes:
            buf = _RESIDENT[idx] = None  # release the old buffer before growing
            buf = _RESIDENT[idx] = torch.empty(nbytes, dtype=torch.uint8, device=device)
        return buf[:nbytes]
    return torch.empty(nbytes, dtype=torch.uint8, device=device)


class resident_workspace:
    """Keeps one workspace buffer on ``device`` for the library calls made inside
    the block (repeated objective evaluations of a fit): calls on the device's
    streams are stream-ordered, so they may share it; do not run concurrent
    streams of library work inside the block."""

    def __init__(self, device=None):
        d = torch.device("cuda") if device is None else torch.device(device)
        self.idx = d.index if d.index is not None else torch.cuda.current_device()

    def __enter__(self):
        self.owner = self.idx not in _RESIDENT
        if self.owner:
            _RESIDENT[self.idx] = None
        return self

    def __exit__(self, *exc):
        if self.owner:
            _RESIDENT.pop(self.idx, None)
        return False
