"""CPU oracle for the portBLAS hot path — TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker.  The product
(``portblas_gb300`` / ``libgbblas.so``) never imports or calls it.

Two oracles live here:

* ``liboracle.so`` — a C restatement (``oracle.c``) of portBLAS's algorithms
  with double-double accumulation, plus reference-order FP32 variants.  Each
  routine cites the portBLAS file:line it follows.
* ``cblas`` — the CBLAS that portBLAS's own tests link
  (``common/include/common/system_reference_blas.hpp``): OpenBLAS, here the
  copy bundled with numpy (``libscipy_openblas64_``, ILP64 symbols).

Parity pinning: portBLAS cannot be built here (no SYCL compiler, empty
``external/py_gen`` submodule), so the oracle is pinned against the
known-answer tests and documented examples of portBLAS's own tests and docs
(``tests/golden``) and cross-checked against the CBLAS oracle.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")

FLT_MAX = float(np.finfo(np.float32).max)
DBL_MAX = float(np.finfo(np.float64).max)


def build(verbose: bool = False) -> str:
    """Compile oracle.c with gcc (OpenMP, no FP contraction)."""
    srcs = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "cpu_baseline.c")]
    os.makedirs(BUILD_DIR, exist_ok=True)
    if os.path.exists(LIB_PATH) and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(s) for s in srcs):
        return LIB_PATH
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", LIB_PATH, *srcs, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        i64, f64, i32 = C.c_int64, C.c_double, C.c_int
        P = C.c_void_p
        L.orc_gemm_f64.argtypes = [i32, i32, i64, i64, i64, f64, P, i64, P, i64, f64, P, i64, i64, P, P, P]
        L.orc_gemm_absscale.argtypes = L.orc_gemm_f64.argtypes
        L.orc_sgemm_reforder.argtypes = [i32, i32, i64, i64, i64, C.c_float, P, i64, P, i64, C.c_float, P, i64, i32]
        L.orc_gemv_f64.argtypes = [C.c_char, i64, i64, f64, P, i64, P, i64, f64, P, i64, P]
        L.orc_asum.argtypes = [i64, P, i64]
        L.orc_asum.restype = f64
        L.orc_dot.argtypes = [i64, P, i64, P, i64]
        L.orc_dot.restype = f64
        L.orc_nrm2.argtypes = [i64, P, i64]
        L.orc_nrm2.restype = f64
        L.orc_iamax.argtypes = [i64, P, i64, i32, f64]
        L.orc_iamax.restype = i64
        L.orc_reduction.argtypes = [i32, i32, P, i64, i64, i64, f64, P]
        L.orc_num_threads.restype = i32
        L.cpu_reduction_f32.argtypes = [i32, i32, P, i64, i64, i64, P]
        L.cpu_reduction_f32.restype = i32
        L.cpu_iamax_f32.argtypes = [i64, P, i32]
        L.cpu_iamax_f32.restype = i64
        _lib = L
    return _lib


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a), dtype=np.float64)


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _tmax(dtype) -> float:
    return FLT_MAX if np.dtype(dtype) == np.float32 else DBL_MAX


# --------------------------------------------------------------- GEMM --
def gemm(ta: bool, tb: bool, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, rows=None, cols=None):
    """FP64 (double-double) C = alpha op(A) op(B) + beta C.

    ``a``, ``b``, ``c`` are flat column-major arrays.  With ``rows``/``cols``
    only those entries are computed (returned as a 1-D array); otherwise the
    full m x n result (Fortran order)."""
    A, B = _f64(a), _f64(b)
    Cm = _f64(c) if c is not None else None
    if rows is not None:
        r = np.ascontiguousarray(rows, dtype=np.int64)
        cc = np.ascontiguousarray(cols, dtype=np.int64)
        out = np.empty(len(r))
        lib().orc_gemm_f64(int(ta), int(tb), m, n, k, alpha, _p(A), lda, _p(B), ldb, beta, _p(Cm), ldc,
                           len(r), _p(r), _p(cc), _p(out))
        return out
    out = np.empty(m * n)
    lib().orc_gemm_f64(int(ta), int(tb), m, n, k, alpha, _p(A), lda, _p(B), ldb, beta, _p(Cm), ldc,
                       -1, None, None, _p(out))
    return out.reshape((m, n), order="F")


def gemm_absscale(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, rows=None, cols=None):
    """|alpha| |op(A)||op(B)| + |beta C| for the same entries as ``gemm``."""
    A, B = _f64(a), _f64(b)
    Cm = _f64(c) if c is not None else None
    if rows is not None:
        r = np.ascontiguousarray(rows, dtype=np.int64)
        cc = np.ascontiguousarray(cols, dtype=np.int64)
        out = np.empty(len(r))
        lib().orc_gemm_absscale(int(ta), int(tb), m, n, k, alpha, _p(A), lda, _p(B), ldb, beta, _p(Cm), ldc,
                                len(r), _p(r), _p(cc), _p(out))
        return out
    out = np.empty(m * n)
    lib().orc_gemm_absscale(int(ta), int(tb), m, n, k, alpha, _p(A), lda, _p(B), ldb, beta, _p(Cm), ldc,
                            -1, None, None, _p(out))
    return out.reshape((m, n), order="F")


def sgemm_reforder(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, mode=0):
    """FP32 GEMM in portBLAS's arithmetic order; returns the new C (flat)."""
    A = np.ascontiguousarray(a, dtype=np.float32)
    B = np.ascontiguousarray(b, dtype=np.float32)
    Cm = np.array(c, dtype=np.float32, copy=True)
    lib().orc_sgemm_reforder(int(ta), int(tb), m, n, k, alpha, _p(A), lda, _p(B), ldb, beta, _p(Cm), ldc, mode)
    return Cm


# --------------------------------------------------------------- GEMV --
def gemv(trans: str, m, n, alpha, a, lda, x, incx, beta, y, incy):
    """Logical y (element i of the view) of alpha op(A) x + beta y in FP64."""
    A, X, Y = _f64(a), _f64(x), _f64(y) if y is not None else None
    tr = trans not in ("n", "N")
    ylen = n if tr else m
    out = np.empty(ylen)
    if Y is None:
        Y = np.zeros(max(1, ylen * abs(incy)))
    lib().orc_gemv_f64(trans.encode()[:1], m, n, alpha, _p(A), lda, _p(X), incx, beta, _p(Y), incy, _p(out))
    return out


def view(vec, n, inc):
    """Logical elements of a strided view (negative inc runs backwards)."""
    v = np.asarray(vec)
    idx = np.arange(n, dtype=np.int64)
    pos = idx * inc if inc >= 0 else (n - 1 - idx) * (-inc)
    return v[pos]


# ------------------------------------------------------------- BLAS-1 --
def asum(n, x, incx) -> float:
    return lib().orc_asum(n, _p(_f64(x)), incx)


def dot(n, x, incx, y, incy) -> float:
    return lib().orc_dot(n, _p(_f64(x)), incx, _p(_f64(y)), incy)


def nrm2(n, x, incx) -> float:
    return lib().orc_nrm2(n, _p(_f64(x)), incx)


def iamax(n, x, incx, dtype=np.float32) -> int:
    return int(lib().orc_iamax(n, _p(_f64(x)), incx, 1, _tmax(dtype)))


def iamin(n, x, incx, dtype=np.float32) -> int:
    return int(lib().orc_iamax(n, _p(_f64(x)), incx, 0, _tmax(dtype)))


# ------------------------------------------------ element-wise BLAS-1 --
def scal(n, alpha, x, incx):
    """x <- alpha*x; alpha == 0 writes zeros (src/interface/blas1_interface.hpp:438-455).
    Returns the whole updated buffer."""
    out = np.array(x, dtype=np.float64, copy=True)
    idx = np.arange(n, dtype=np.int64)
    pos = idx * incx if incx >= 0 else (n - 1 - idx) * (-incx)
    out[pos] = 0.0 if alpha == 0 else alpha * out[pos]
    return out


def axpy(n, alpha, x, incx, y, incy):
    """y <- alpha*x + y on strided views; returns the whole updated y."""
    out = np.array(y, dtype=np.float64, copy=True)
    idx = np.arange(n, dtype=np.int64)
    py = idx * incy if incy >= 0 else (n - 1 - idx) * (-incy)
    out[py] = alpha * view(x, n, incx) + out[py]
    return out


def copy(n, x, incx, y, incy):
    out = np.array(y, dtype=np.float64, copy=True)
    idx = np.arange(n, dtype=np.int64)
    py = idx * incy if incy >= 0 else (n - 1 - idx) * (-incy)
    out[py] = view(x, n, incx)
    return out


def sdsdot(n, sb, x, incx, y, incy):
    """sb + dot(x, y); n == 0 gives sb (src/interface/blas1_interface.hpp:150-177)."""
    return float(sb) + (dot(n, x, incx, y, incy) if n > 0 else 0.0)


def omatcopy(trans, m, n, alpha, a, ld_in, out, ld_out):
    """out <- alpha*op(in) (include/interface/extension_interface.h:175-198);
    returns the whole updated out buffer."""
    A = np.asarray(a, dtype=np.float64)
    res = np.array(out, dtype=np.float64, copy=True)
    for j in range(n):
        col = alpha * A[j * ld_in: j * ld_in + m]
        if trans in ("n", "N"):
            res[j * ld_out: j * ld_out + m] = col
        else:
            res[j + np.arange(m) * ld_out] = col
    return res


def symm(side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc):
    """SYMM from the referenced triangle of A (one triangle mirrored), then
    the double-double GEMM oracle (m x n result, Fortran order)."""
    na = m if side in ("l", "L") else n
    A = np.asarray(a, dtype=np.float64)
    full = np.empty((na, na))
    for j in range(na):
        for i in range(na):
            direct = (i <= j) if uplo in ("u", "U") else (i >= j)
            full[i, j] = A[i + j * lda] if direct else A[j + i * lda]
    F = full.ravel(order="F")
    if side in ("l", "L"):
        return gemm(False, False, m, n, m, alpha, F, na, b, ldb, beta, c, ldc)
    return gemm(False, False, m, n, n, alpha, b, ldb, F, na, beta, c, ldc)


# ---------------------------------------------------------- reduction --
OPS = {"add": 0, "product": 1, "max": 2, "min": 3, "abs_add": 4, "mean": 5}
DIMS = {"inner": 0, "outer": 1}


def reduction(op: str, dim: str, inp, ld, rows, cols, dtype=np.float32):
    nout = cols if dim == "inner" else rows
    out = np.empty(nout)
    lib().orc_reduction(OPS[op], DIMS[dim], _p(_f64(inp)), ld, rows, cols, _tmax(dtype), _p(out))
    return out


# ----------------------------------------- timed CPU baseline (cpu_baseline.c) --
def cpu_reduction_add(dim: str, inp, ld, rows, cols, out=None):
    """FP32 OpenMP restatement of portBLAS's Reduction kernel (AddOperator);
    the timed CPU baseline, not a checker.  ``inp`` must be float32."""
    a = np.asarray(inp)
    assert a.dtype == np.float32 and a.flags.c_contiguous
    nout = cols if dim == "inner" else rows
    if out is None:
        out = np.empty(nout, np.float32)
    if lib().cpu_reduction_f32(0, DIMS[dim], _p(a), ld, rows, cols, _p(out)) != 0:
        raise ValueError("cpu_reduction_f32: unsupported operator")
    return out


def cpu_iamax(x, is_min: bool = False) -> int:
    """OpenMP first-index max/min |x| over a float32 vector (timed CPU baseline)."""
    a = np.asarray(x)
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return int(lib().cpu_iamax_f32(len(a), _p(a), int(is_min)))


def num_threads() -> int:
    return int(lib().orc_num_threads())


# ------------------------------------------------------- CBLAS oracle --
class CBlas:
    """numpy's bundled OpenBLAS through its ILP64 CBLAS symbols."""

    ColMajor, NoTrans, Trans = 102, 111, 112

    def __init__(self):
        import numpy as _np
        libdir = os.path.join(os.path.dirname(os.path.dirname(_np.__file__)), "numpy.libs")
        cands = sorted(glob.glob(os.path.join(libdir, "libscipy_openblas64_*.so*")))
        if not cands:
            raise OSError(f"no bundled OpenBLAS under {libdir}")
        self.path = cands[0]
        L = C.CDLL(self.path)
        i64, i32, f32, f64, P = C.c_int64, C.c_int, C.c_float, C.c_double, C.c_void_p
        L.scipy_cblas_sgemm64_.argtypes = [i32, i32, i32, i64, i64, i64, f32, P, i64, P, i64, f32, P, i64]
        L.scipy_cblas_dgemm64_.argtypes = [i32, i32, i32, i64, i64, i64, f64, P, i64, P, i64, f64, P, i64]
        L.scipy_cblas_sgemv64_.argtypes = [i32, i32, i64, i64, f32, P, i64, P, i64, f32, P, i64]
        L.scipy_cblas_sasum64_.argtypes = [i64, P, i64]
        L.scipy_cblas_sasum64_.restype = f32
        L.scipy_cblas_snrm264_.argtypes = [i64, P, i64]
        L.scipy_cblas_snrm264_.restype = f32
        L.scipy_cblas_sdot64_.argtypes = [i64, P, i64, P, i64]
        L.scipy_cblas_sdot64_.restype = f32
        L.scipy_cblas_isamax64_.argtypes = [i64, P, i64]
        L.scipy_cblas_isamax64_.restype = i64
        L.scipy_cblas_saxpy64_.argtypes = [i64, f32, P, i64, P, i64]
        L.scipy_cblas_sscal64_.argtypes = [i64, f32, P, i64]
        L.scipy_cblas_scopy64_.argtypes = [i64, P, i64, P, i64]
        L.scipy_cblas_sdsdot64_.argtypes = [i64, f32, P, i64, P, i64]
        L.scipy_cblas_sdsdot64_.restype = f32
        L.scipy_cblas_ssymm64_.argtypes = [i32, i32, i32, i64, i64, f32, P, i64, P, i64, f32, P, i64]
        L.scipy_cblas_somatcopy64_.argtypes = [i32, i32, i64, i64, f32, P, i64, P, i64]
        for nm in ("scipy_openblas_set_num_threads64_", "scipy_openblas_get_num_threads64_"):
            if not hasattr(L, nm):
                raise OSError(f"{nm} missing from {self.path}")
        L.scipy_openblas_set_num_threads64_.argtypes = [i32]
        L.scipy_openblas_get_num_threads64_.restype = i32
        self.L = L

    def set_threads(self, n: int) -> None:
        self.L.scipy_openblas_set_num_threads64_(int(n))

    def threads(self) -> int:
        return int(self.L.scipy_openblas_get_num_threads64_())

    def sgemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
        t = lambda f: self.Trans if f else self.NoTrans
        self.L.scipy_cblas_sgemm64_(self.ColMajor, t(ta), t(tb), m, n, k, alpha, _p(a), lda, _p(b), ldb, beta,
                                    _p(c), ldc)

    def dgemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
        t = lambda f: self.Trans if f else self.NoTrans
        self.L.scipy_cblas_dgemm64_(self.ColMajor, t(ta), t(tb), m, n, k, alpha, _p(a), lda, _p(b), ldb, beta,
                                    _p(c), ldc)

    def sgemv(self, trans, m, n, alpha, a, lda, x, incx, beta, y, incy):
        t = self.NoTrans if trans in ("n", "N") else self.Trans
        self.L.scipy_cblas_sgemv64_(self.ColMajor, t, m, n, alpha, _p(a), lda, _p(x), incx, beta, _p(y), incy)

    def sasum(self, n, x, incx):
        return self.L.scipy_cblas_sasum64_(n, _p(x), incx)

    def snrm2(self, n, x, incx):
        return self.L.scipy_cblas_snrm264_(n, _p(x), incx)

    def sdot(self, n, x, incx, y, incy):
        return self.L.scipy_cblas_sdot64_(n, _p(x), incx, _p(y), incy)

    def isamax(self, n, x, incx):
        return int(self.L.scipy_cblas_isamax64_(n, _p(x), incx))

    def saxpy(self, n, alpha, x, incx, y, incy):
        self.L.scipy_cblas_saxpy64_(n, alpha, _p(x), incx, _p(y), incy)

    def sscal(self, n, alpha, x, incx):
        self.L.scipy_cblas_sscal64_(n, alpha, _p(x), incx)

    def scopy(self, n, x, incx, y, incy):
        self.L.scipy_cblas_scopy64_(n, _p(x), incx, _p(y), incy)

    def sdsdot(self, n, sb, x, incx, y, incy):
        return self.L.scipy_cblas_sdsdot64_(n, sb, _p(x), incx, _p(y), incy)

    Left, Right, Upper, Lower = 141, 142, 121, 122

    def ssymm(self, side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc):
        sd = self.Left if side in ("l", "L") else self.Right
        ul = self.Upper if uplo in ("u", "U") else self.Lower
        self.L.scipy_cblas_ssymm64_(self.ColMajor, sd, ul, m, n, alpha, _p(a), lda, _p(b), ldb, beta, _p(c), ldc)

    def somatcopy(self, trans, m, n, alpha, a, lda, b, ldb):
        """OpenBLAS extension: b <- alpha * op(a), a is m x n (column-major)."""
        t = self.NoTrans if trans in ("n", "N") else self.Trans
        self.L.scipy_cblas_somatcopy64_(self.ColMajor, t, m, n, alpha, _p(a), lda, _p(b), ldb)

    @staticmethod
    def isamin(n, x, incx):
        """portBLAS's test-side iamin: first strict minimum of |x|
        (common/include/common/system_reference_blas.hpp:91-101)."""
        v = np.abs(np.asarray(x)[: n * incx: incx]) if incx > 0 else np.abs(np.asarray(x))[:0]
        return int(np.argmin(v)) if len(v) else 0
