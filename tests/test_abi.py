"""Host-side checks of the C ABI (no GPU needed): the library loads, exports
every entry point include/gbblas.h declares, and rejects a null handle."""
import ctypes as C
import os
import subprocess

import pytest

from portblas_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    build.build()
    return _lib.load()


def test_header_declares_hot_path():
    names = set(_lib.parse_header())
    for op in ("sgemm", "dgemm", "sgemm_batched", "sgemm_strided_batched", "sgemv", "dgemv", "sasum", "snrm2",
               "sdot", "ddot", "isamax", "isamin", "sreduction", "gemm_grouped", "handle_create"):
        assert f"gbblas_{op}" in names


def test_library_exports_every_declared_symbol(L):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True, check=True)
    exported = {ln.split()[-1] for ln in out.stdout.splitlines() if ln.strip()}
    missing = [n for n in _lib.parse_header() if n not in exported]
    assert not missing, missing
    # nothing beyond the C ABI leaks out (hidden visibility)
    extra = [n for n in exported if n.startswith("_Z") and "gb" in n]
    assert not extra, extra[:5]


def test_status_strings(L):
    assert L.gbblas_status_string(0) == b"success"
    assert L.gbblas_status_string(1) == b"invalid argument"
    assert L.gbblas_status_string(4) == b"device wait timed out"


def test_null_handle_is_rejected_without_touching_the_gpu(L):
    x = C.c_float()
    assert L.gbblas_sasum(None, 10, None, 1, C.addressof(x)) == 6
    assert b"null handle" in L.gbblas_last_error()
    assert L.gbblas_sgemm(None, b"n", b"n", 4, 4, 4, 1.0, None, 4, None, 4, 0.0, None, 4) == 6
    assert L.gbblas_sgemv(None, b"n", 4, 4, 1.0, None, 4, None, 1, 0.0, None, 1) == 6
    assert L.gbblas_sreduction(None, 0, 0, None, 4, None, 4, 4) == 6
    assert L.gbblas_wait(None) == 6
    assert L.gbblas_handle_destroy(None) == 0


def test_handle_create_rejects_null_out(L):
    assert L.gbblas_handle_create(None, None) == 1


def test_python_mirror_names_follow_portblas():
    from portblas_gb300 import blas
    for fn in ("_gemm", "_gemm_batched", "_gemm_strided_batched", "_gemv", "_asum", "_nrm2", "_dot", "_iamax",
               "_iamin"):
        assert callable(getattr(blas, fn))
    assert callable(blas.extension._reduction)
    assert blas.reduction_dim_t.inner == 0 and blas.reduction_dim_t.outer == 1
    assert blas.gemm_batch_type_t.strided == 0


def test_product_path_does_not_import_the_oracle():
    import sys
    import importlib
    for m in [k for k in sys.modules if k == "oracle" or k.startswith("oracle.")]:
        del sys.modules[m]
    import portblas_gb300.blas  # noqa: F401
    importlib.reload(portblas_gb300.blas)
    assert "oracle" not in sys.modules
    src_dir = os.path.join(ROOT, "portblas_gb300")
    for dp, _, fs in os.walk(src_dir):
        for f in fs:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                text = open(os.path.join(dp, f)).read()
                assert "import oracle" not in text and "liboracle" not in text, f
