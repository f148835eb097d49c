"""GPU: the allocation-free marginal log-likelihood entry point.

gpk_conjugate_mll_noalloc serves callers that cannot allocate device memory
(custom calls that receive no workspace, hosts that forbid allocation after
start-up): its scratch is a fixed 8 MiB
device array inside the library, so it takes no workspace and handles
n <= 512.  This test calls it through the C ABI and compares it with
gpk_conjugate_mll (which takes caller-allocated workspace) on the same inputs,
twice in a row with different data, since every call reuses the same array.

This file is named to be collected last, so a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

from gpjax_gb300 import _lib

pytestmark = pytest.mark.gpu

GPK_ERR_UNSUPPORTED = 6


def _inputs(seed, n, d, kind):
    rng = np.random.default_rng(seed)
    x = torch.as_tensor(rng.standard_normal((n, d)), device="cuda")
    y = torch.as_tensor(np.sin(rng.standard_normal(n)), device="cuda")
    ls = np.exp(rng.uniform(np.log(0.5), np.log(2.0), d))
    theta = torch.as_tensor(np.concatenate([ls, [1.3, 0.2, 0.1]]), device="cuda")
    return x, y, theta


def _with_workspace(kind, x, y, theta, d):
    lib = _lib.lib()
    n = x.shape[0]
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    grad = torch.empty(d + 3, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = _lib.workspace(lib.gpk_conjugate_mll_workspace_bytes(n, d, _lib.PREC_FP64), x.device)
    st = lib.gpk_conjugate_mll(kind, n, d, x.data_ptr(), d, y.data_ptr(), theta.data_ptr(), d,
                               1e-6, _lib.PREC_FP64, 1, out.data_ptr(), grad.data_ptr(),
                               info.data_ptr(), ws.data_ptr(), ws.numel(), _lib.stream_ptr())
    assert st == 0
    return out, grad, info


def _no_alloc(kind, x, y, theta, d):
    lib = _lib.lib()
    n = x.shape[0]
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    grad = torch.empty(d + 3, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = lib.gpk_conjugate_mll_noalloc(kind, n, d, x.data_ptr(), d, y.data_ptr(),
                                       theta.data_ptr(), d, 1e-6, 1, out.data_ptr(),
                                       grad.data_ptr(), info.data_ptr(), _lib.stream_ptr())
    assert st == 0
    return out, grad, info


def test_no_alloc_matches_workspace_entry_point_twice(cuda_lib):
    assert _lib.lib().gpk_conjugate_mll_noalloc_max_n() == 512
    # two calls in a row with different sizes, kernels and data: the second
    # call runs over whatever the first one left in the shared scratch array
    for seed, n, d, kind in ((1, 512, 8, _lib.MATERN52), (2, 300, 3, _lib.RBF)):
        x, y, theta = _inputs(seed, n, d, kind)
        ref, gref, iref = _with_workspace(kind, x, y, theta, d)
        val, g, info = _no_alloc(kind, x, y, theta, d)
        torch.cuda.synchronize()
        assert int(info.item()) == 0 and int(iref.item()) == 0
        r, v = float(ref.item()), float(val.item())
        # same float64 algorithm: the float64 parity tolerances of the other tests
        assert abs(v - r) <= 1e-10 * abs(r), (v, r)
        assert torch.allclose(g, gref, rtol=1e-7, atol=1e-9), (g, gref)


def test_no_alloc_takes_no_device_memory(cuda_lib):
    """After a first call on the device (which loads the library's kernels),
    further calls change neither torch's allocation count nor the device's
    free memory."""
    x, y, theta = _inputs(3, 256, 4, _lib.RBF)
    _no_alloc(_lib.RBF, x, y, theta, 4)
    torch.cuda.synchronize()
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    grad = torch.empty(7, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib = _lib.lib()
    alloc0, free0 = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0]
    for _ in range(2):
        st = lib.gpk_conjugate_mll_noalloc(_lib.RBF, 256, 4, x.data_ptr(), 4, y.data_ptr(),
                                           theta.data_ptr(), 4, 1e-6, 1, out.data_ptr(),
                                           grad.data_ptr(), info.data_ptr(), _lib.stream_ptr())
        assert st == 0
    torch.cuda.synchronize()
    assert int(info.item()) == 0 and np.isfinite(float(out.item()))
    assert torch.cuda.memory_allocated() == alloc0
    assert torch.cuda.mem_get_info()[0] == free0


def test_no_alloc_refuses_sizes_beyond_its_scratch(cuda_lib):
    lib = _lib.lib()
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: the size check fails first
    st = lib.gpk_conjugate_mll_noalloc(_lib.RBF, 513, 2, fake, 2, fake, fake, 1, 1e-6, 1, fake,
                                       fake, fake, None)
    assert st == GPK_ERR_UNSUPPORTED
    assert b"unsupported" in lib.gpk_status_string(st)
