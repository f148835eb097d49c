"""The JAX custom-call layer on CPU: the module imports and reports itself
unavailable without jax; its kernel codes are the C ABI's; the handler source
type-checks against include/gpk.h (through a compile-only stand-in for
jaxlib's FFI header) and defines every target the module registers."""
import os
import re
import shutil
import subprocess

import pytest

import gpjax_gb300.jax_ffi as gfx
from gpjax_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_imports_and_reports_availability():
    try:
        import jax  # noqa: F401
        have = hasattr(jax, "ffi")
    except ImportError:
        have = False
    assert gfx.available() == have
    if not have:
        with pytest.raises(RuntimeError, match="needs jax"):
            gfx.conjugate_mll(None, None)


def test_kernel_codes_match_the_c_abi():
    assert gfx.KINDS == {"RBF": _lib.RBF, "Matern32": _lib.MATERN32, "Matern52": _lib.MATERN52,
                         "Matern12": _lib.MATERN12, "RationalQuadratic": _lib.RATIONAL_QUADRATIC}
    assert gfx.PRECISIONS == {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}


def test_every_registered_target_is_defined():
    src = open(gfx.SRC).read()
    defined = set(re.findall(r"XLA_FFI_DEFINE_HANDLER_SYMBOL\((\w+),", src))
    assert set(gfx.TARGETS.values()) == defined


def test_handlers_type_check_against_the_header():
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda_inc = "/usr/local/cuda/include"
    if not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("no CUDA headers")
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Werror",
                        f"-I{os.path.join(ROOT, 'tests', 'ffi_stub')}",
                        f"-I{os.path.join(ROOT, 'include')}", f"-I{cuda_inc}", gfx.SRC],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
