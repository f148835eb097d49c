"""CPU: the C-ABI library loads, exports every entry point that include/gpk.h
declares, and its host-only paths (workspace queries, argument validation)
behave.  No compute call is made, so no GPU is needed."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(gpk_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("gpk_conjugate_mll", "gpk_gram", "gpk_cross_covariance",
                     "gpk_lower_cholesky", "gpk_solve_triangular", "gpk_predict"):
        assert required in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_header(built_lib):
    from gpjax_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_version_and_status_strings(built_lib):
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    assert lib.gpk_version() >= 100
    assert lib.gpk_status_string(0) == b"ok"
    assert b"workspace" in lib.gpk_status_string(3)


def test_workspace_queries(built_lib):
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    a = lib.gpk_conjugate_mll_workspace_bytes(16384, 8, _lib.PREC_MIXED)
    b = lib.gpk_conjugate_mll_workspace_bytes(16384, 8, _lib.PREC_FP64)
    # mixed: the float32 input and its TF32 hi/lo copy plus TF32 hi/lo pairs of L,
    # L^-1 and L^-T (9 n x n), the float16 hi/lo copy of L^-T (1 n x n), the
    # per-depth T^T scratch (~2/3 n x n) and the float16 operand copies of the
    # wide recursion nodes (~1.3 n x n)
    assert 11 * 16384 * 16384 * 4 < a < 14 * 16384 * 16384 * 4
    # float64: factor, inverse and transposed inverse plus scratch
    assert 3 * 16384 * 16384 * 8 < b < 5 * 16384 * 16384 * 8
    assert lib.gpk_predict_workspace_bytes(2048, 512, 4, _lib.PREC_FP64) > 0
    assert lib.gpk_solve_triangular_workspace_bytes(100, 3, _lib.F64) > 0


@pytest.mark.parametrize("kind,n,d,n_ls,prec", [
    (7, 10, 2, 1, 0),      # unknown kernel
    (0, -1, 2, 1, 0),      # negative n
    (0, 10, 0, 1, 0),      # d = 0
    (0, 10, 3, 2, 0),      # n_ls neither 1 nor d
    (0, 10, 3, 3, 9),      # unknown precision
    (0, 10, 99, 1, 0),     # d above the register limit
])
def test_mll_rejects_bad_arguments(built_lib, kind, n, d, n_ls, prec):
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    st = lib.gpk_conjugate_mll(kind, n, d, None, max(d, 1), None, None, n_ls, 1e-6, prec, 1,
                               None, None, None, None, 0, None)
    assert st == 1  # GPK_ERR_BAD_ARG, returned before any device work


def test_mll_rejects_small_workspace(built_lib):
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: the size check fails first
    st = lib.gpk_conjugate_mll(0, 100, 2, fake, 2, fake, fake, 1, 1e-6, 0, 1, fake, fake, fake,
                               fake, 16, None)
    assert st == 3  # GPK_ERR_WORKSPACE


def test_cross_covariance_rejects_bad_arguments(built_lib):
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    assert lib.gpk_cross_covariance(5, 3, 3, 2, None, 2, None, 2, None, 1, 0, None, 3, None) == 1
    assert lib.gpk_cross_covariance(0, 3, 3, 2, None, 1, None, 2, None, 1, 0, None, 3, None) == 1


def test_product_has_no_cpu_fallback():
    """The package never imports the oracle, and fails loudly without CUDA."""
    import subprocess
    import sys
    code = ("import sys, gpjax_gb300, torch\n"
            "assert not any(m.startswith('oracle') for m in sys.modules)\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pkg = os.path.join(ROOT, "gpjax_gb300")
    for f in os.listdir(pkg):
        if f.endswith(".py"):
            assert "oracle" not in open(os.path.join(pkg, f)).read().replace("oracle is", ""), f


def test_batched_mll_rejects_bad_arguments(built_lib):
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    n = (ctypes.c_int64 * 1)(100)
    d = (ctypes.c_int * 1)(2)
    assert lib.gpk_conjugate_mll_batched_workspace_bytes(1, n, d) > 256
    nul = [None] * 5
    # (count, kind, n, d, x, ldx, y, theta, n_ls, jitter, want_grad, out_mll, out_grad,
    #  info, workspace, workspace_bytes, stream)
    assert lib.gpk_conjugate_mll_batched(-1, None, n, d, *nul, 1e-6, 1, None, None, None, None,
                                         0, None) == 1
    # null per-instance arrays are refused before any device work
    assert lib.gpk_conjugate_mll_batched(1, None, n, d, *nul, 1e-6, 1, None, None, None, None,
                                         0, None) == 1


def test_batch_plan_rejects_bad_arguments(built_lib):
    """Plan creation checks every instance on the host before touching the
    device; a null plan is refused by execute and harmless elsewhere."""
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    P = ctypes.c_void_p(0x1000)
    ptr1 = (ctypes.c_void_p * 1)(P)
    i32 = lambda *v: (ctypes.c_int * len(v))(*v)
    i64 = lambda *v: (ctypes.c_int64 * len(v))(*v)
    out = ctypes.c_void_p()

    def create(count=1, kind=0, n=100, d=2, ldx=2, nls=2, jitter=1e-6):
        return lib.gpk_batch_plan_create(count, i32(kind), i64(n), i32(d), ptr1, i64(ldx), ptr1,
                                         ptr1, i32(nls), jitter, 1, ptr1, ptr1, P, 0,
                                         ctypes.byref(out))
    assert create(count=0) == 1
    assert create(kind=7) == 1
    assert create(n=0) == 1
    assert create(ldx=1) == 1
    assert create(nls=3) == 1
    assert create(jitter=-1.0) == 1
    assert create(n=4097) == 6          # GPK_ERR_UNSUPPORTED: one CTA per instance up to 4096
    assert create(d=17, ldx=17, nls=17) == 6
    assert out.value is None
    assert lib.gpk_batch_plan_create(1, i32(0), i64(100), i32(2), ptr1, i64(2), ptr1, ptr1,
                                     i32(2), 1e-6, 1, ptr1, ptr1, P, 0, None) == 1
    assert lib.gpk_batch_plan_workspace_bytes(None) == 0
    assert lib.gpk_batch_plan_config(None, 100) == -1
    assert lib.gpk_batch_plan_execute(None, P, 1 << 20, None) == 1
    assert lib.gpk_batch_plan_destroy(None) == 0
    assert lib.gpk_batch_plan_config_count() == 3
    assert lib.gpk_batch_plan_force_config(None, 0) == 1
    assert lib.gpk_batch_plan_selftest_stall(None, 0) == 1


# ---------------------------------------------------------------------------
# Argument checks of the remaining entry points: every case below is refused
# on the host before any device work (fake pointers are never dereferenced)
# ---------------------------------------------------------------------------
_P = ctypes.c_void_p(0x1000)


def test_kernel_entry_points_reject_bad_arguments(built_lib):
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    # gram / diagonal: unknown kernel, ldx < d, n_ls neither 1 nor d, null output
    assert lib.gpk_gram(9, 4, 2, _P, 2, _P, 1, 0, _P, 4, None) == 1
    assert lib.gpk_gram(0, 4, 2, _P, 1, _P, 1, 0, _P, 4, None) == 1
    assert lib.gpk_gram(0, 4, 3, _P, 3, _P, 2, 0, _P, 4, None) == 1
    assert lib.gpk_gram(0, 4, 2, _P, 2, _P, 1, 0, None, 4, None) == 1
    assert lib.gpk_gram(0, 0, 2, None, 2, None, 1, 0, None, 0, None) == 0  # empty: no work
    assert lib.gpk_diagonal(0, 4, 2, _P, 1, _P, 1, _P, None) == 1
    assert lib.gpk_diagonal(0, 4, 2, None, 2, _P, 1, _P, None) == 1
    # cross-covariance cotangent: m < 0, ldy < d, missing outputs, small workspace
    ws = lib.gpk_cross_covariance_vjp_workspace_bytes(5, 6, 2)
    assert ws > 0
    assert lib.gpk_cross_covariance_vjp(0, 5, -1, 2, _P, 2, _P, 2, _P, 1, _P, 6, _P, None, None,
                                        _P, ws, None) == 1
    assert lib.gpk_cross_covariance_vjp(0, 5, 6, 2, _P, 2, _P, 1, _P, 1, _P, 6, _P, None, None,
                                        _P, ws, None) == 1
    assert lib.gpk_cross_covariance_vjp(0, 5, 6, 2, _P, 2, _P, 2, _P, 1, _P, 6, None, None,
                                        None, _P, ws, None) == 1
    assert lib.gpk_cross_covariance_vjp(0, 5, 6, 2, _P, 2, _P, 2, _P, 1, _P, 6, _P, None, None,
                                        _P, 8, None) == 3


def test_linalg_entry_points_reject_bad_arguments(built_lib):
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    info = _P
    assert lib.gpk_lower_cholesky(-1, _lib.F64, _P, 4, None, info, None) == 1
    assert lib.gpk_lower_cholesky(8, _lib.F64, _P, 4, None, info, None) == 1   # lda < n
    assert lib.gpk_lower_cholesky(8, _lib.F64, _P, 8, None, None, None) == 1   # info missing
    assert lib.gpk_lower_cholesky(8, 7, _P, 8, None, info, None) == 1          # unknown dtype
    ws = lib.gpk_solve_triangular_workspace_bytes(8, 3, _lib.F64)
    assert lib.gpk_solve_triangular(8, 3, _lib.F64, _P, 8, _P, 2, _P, ws, None) == 1  # ldb < nrhs
    assert lib.gpk_solve_triangular(8, 3, _lib.F64, _P, 8, _P, 3, _P, 8, None) == 3
    assert lib.gpk_solve_triangular(8, 3, 7, _P, 8, _P, 3, _P, ws, None) == 1
    assert lib.gpk_solve_triangular(0, 3, _lib.F64, None, 0, None, 3, None, 0, None) == 0
    assert lib.gpk_logdet_triangular(8, _lib.F64, None, 8, _P, None) == 1
    assert lib.gpk_logdet_triangular(8, _lib.F64, _P, 4, _P, None) == 1
    assert lib.gpk_logdet_triangular(8, 7, _P, 8, _P, None) == 1


def test_objective_entry_points_reject_bad_arguments(built_lib):
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    # collapsed ELBO: (kind, n, m, d, x, ldx, y, z, ldz, theta, n_ls, jitter, precision,
    # want_grad, out_elbo, out_grad, out_grad_z, info, workspace, workspace_bytes, stream)
    ws = lib.gpk_collapsed_elbo_workspace_bytes(100, 10, 2, _lib.PREC_MIXED)
    ok = [0, 100, 10, 2, _P, 2, _P, _P, 2, _P, 1, 1e-6, _lib.PREC_MIXED, 1, _P, _P, _P, _P, _P,
          ws, None]

    def elbo(**kw):
        a = list(ok)
        for k, v in kw.items():
            a[int(k[1:])] = v
        return lib.gpk_collapsed_elbo(*a)

    assert elbo(a0=7) == 1                # unknown kernel
    assert elbo(a2=20000) == 1            # m above the inducing-point bound
    assert elbo(a3=17) == 1               # d above the SGPR input bound
    assert elbo(a10=3) == 1               # n_ls neither 1 nor d
    assert elbo(a12=5) == 1               # unknown precision
    assert elbo(a15=None) == 1            # gradient wanted, no output
    assert elbo(a19=16) == 3              # workspace too small
    # predict: (kind, n, t, d, x, ldx, y, xt, ldxt, theta, n_ls, jitter, prior_jitter,
    # precision, mean, var, cov, ldcov, info, workspace, workspace_bytes, stream)
    pws = lib.gpk_predict_workspace_bytes(50, 5, 2, _lib.PREC_FP64)
    assert lib.gpk_predict(0, 0, 5, 2, _P, 2, _P, _P, 2, _P, 1, 1e-6, 1e-6, 0, _P, _P, None, 0,
                           _P, _P, pws, None) == 1                       # n = 0
    assert lib.gpk_predict(0, 50, 5, 2, _P, 2, _P, _P, 1, _P, 1, 1e-6, 1e-6, 0, _P, _P, None, 0,
                           _P, _P, pws, None) == 1                       # ldxt < d
    assert lib.gpk_predict(0, 50, 5, 2, _P, 2, _P, _P, 2, _P, 1, 1e-6, 1e-6, 0, _P, _P, _P, 3,
                           _P, _P, pws, None) == 1                       # ldcov < t
    assert lib.gpk_predict(0, 50, 0, 2, None, 2, None, None, 2, None, 1, 1e-6, 1e-6, 0, None,
                           None, None, 0, None, None, 0, None) == 0      # t = 0: no work
    # the allocation-free MLL: sizes past its static scratch are unsupported
    big = lib.gpk_conjugate_mll_noalloc_max_n() + 1
    assert lib.gpk_conjugate_mll_noalloc(0, big, 2, _P, 2, _P, _P, 1, 1e-6, 1, _P, _P, _P,
                                         None) == 6
    assert lib.gpk_conjugate_mll_noalloc(0, 10, 2, _P, 2, _P, None, 1, 1e-6, 1, _P, _P, _P,
                                         None) == 1
    # leave-one-out objective: argument checks before any device work
    lws = lib.gpk_conjugate_loocv_workspace_bytes(50, 2)
    assert lws > 0
    assert lib.gpk_conjugate_loocv(5, 50, 2, _P, 2, _P, _P, 1, 1e-6, 1, _P, _P, _P, _P, lws,
                                   None) == 1                            # unknown kernel
    assert lib.gpk_conjugate_loocv(0, 50, 2, _P, 1, _P, _P, 1, 1e-6, 1, _P, _P, _P, _P, lws,
                                   None) == 1                            # ldx < d
    assert lib.gpk_conjugate_loocv(0, 50, 2, _P, 2, _P, _P, 3, 1e-6, 1, _P, _P, _P, _P, lws,
                                   None) == 1                            # n_ls not 1 or d
    assert lib.gpk_conjugate_loocv(0, 50, 2, _P, 2, _P, _P, 1, 1e-6, 1, _P, _P, _P, _P, lws - 1,
                                   None) == 3                            # workspace too small
    # d past the library-wide bound (32) is a bad argument, as for gpk_conjugate_mll
    assert lib.gpk_conjugate_mll_noalloc(0, 10, 33, _P, 33, _P, _P, 1, 1e-6, 1, _P, _P, _P,
                                         None) == 1
    assert lib.gpk_conjugate_mll_noalloc(0, 10, 32, _P, 31, _P, _P, 1, 1e-6, 1, _P, _P, _P,
                                         None) == 1                      # ldx < d


def test_gemm_entry_point_rejects_bad_arguments(built_lib):
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    ws = lib.gpk_gemm_tf32x3_workspace_bytes(64, 64, 32)
    # (M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lower_only, err_flag, workspace, bytes, stream)
    assert lib.gpk_gemm_tf32x3(-1, 64, 32, 1.0, _P, 32, _P, 32, 0.0, _P, 64, 0, None, _P, ws,
                               None) == 1
    assert lib.gpk_gemm_tf32x3(64, 64, 32, 1.0, _P, 16, _P, 32, 0.0, _P, 64, 0, None, _P, ws,
                               None) == 1                                  # lda < K
    assert lib.gpk_gemm_tf32x3(64, 48, 32, 1.0, _P, 32, _P, 32, 0.0, _P, 64, 1, None, _P, ws,
                               None) == 1                                  # lower_only, M != N
    assert lib.gpk_gemm_tf32x3(64, 64, 32, 1.0, _P, 32, _P, 32, 0.0, _P, 64, 0, None, _P, 8,
                               None) == 3
    assert lib.gpk_gemm_tf32x3(0, 64, 32, 1.0, None, 32, None, 32, 0.0, None, 64, 0, None, None,
                               0, None) == 0                               # empty product


def test_header_is_plain_c_and_links(built_lib, tmp_path):
    """include/gpk.h compiles as C (no C++ or torch types across the boundary),
    and a C program links libgpk.so and calls its host-only entry points."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    cuda_inc = "/usr/local/cuda/include"
    if gcc is None or not os.path.isdir(cuda_inc):
        pytest.skip("gcc or the CUDA headers are not available")
    src = tmp_path / "probe.c"
    src.write_text(
        '#include <stdio.h>\n#include <string.h>\n#include "gpk.h"\n'
        "int main(void) {\n"
        "  if (gpk_version() <= 0) return 1;\n"
        "  if (strlen(gpk_status_string(GPK_ERR_BAD_ARG)) == 0) return 2;\n"
        "  if (gpk_conjugate_mll(7, 10, 2, NULL, 2, NULL, NULL, 1, 1e-6, GPK_PREC_FP64, 1,\n"
        "                        NULL, NULL, NULL, NULL, 0, NULL) != GPK_ERR_BAD_ARG) return 3;\n"
        '  printf("ok %d\\n", gpk_version());\n'
        "  return 0;\n}\n")
    exe = tmp_path / "probe"
    libdir = os.path.dirname(str(built_lib))
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-x", "c", str(src), "-o", str(exe),
                        f"-I{os.path.join(ROOT, 'include')}", f"-I{cuda_inc}", f"-L{libdir}",
                        "-lgpk", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True)
    assert run.returncode == 0 and run.stdout.startswith("ok"), (run.returncode, run.stderr)


def test_workspace_queries_grow_with_the_problem(built_lib):
    """Layout sanity: every workspace query is monotone in the problem size
    (the mixed MLL gains per-depth float16 operand copies from n = 4096 on)."""
    from gpjax_gb300 import _lib
    lib = _lib.lib()
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
        sizes = [lib.gpk_conjugate_mll_workspace_bytes(n, 8, prec)
                 for n in (100, 128, 129, 1000, 2048, 4095, 4096, 4097, 8192, 16384)]
        assert all(b >= a for a, b in zip(sizes, sizes[1:])), (prec, sizes)
        el = [lib.gpk_collapsed_elbo_workspace_bytes(n, m, 4, prec)
              for n, m in ((1000, 10), (1000, 100), (5000, 100), (9000, 100), (9000, 1024))]
        assert all(b >= a for a, b in zip(el, el[1:])), (prec, el)
        pr = [lib.gpk_predict_workspace_bytes(n, t, 4, prec)
              for n, t in ((100, 10), (100, 100), (1000, 100), (4000, 512))]
        assert all(b >= a for a, b in zip(pr, pr[1:])), (prec, pr)
    # the float16 copies of the wide nodes: present from n_pad = 4096 (halves of 2048)
    mixed = {n: lib.gpk_conjugate_mll_workspace_bytes(n, 8, _lib.PREC_MIXED) for n in (3968, 4096)}
    assert mixed[4096] - mixed[3968] > 16 * 2048 * 2048
