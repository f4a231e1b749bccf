"""Python mirror of portBLAS's ``blas::`` interface for the hot path.

Same function names, argument order and meaning as the C++ templates in
portBLAS's ``include/interface/blas{1,2,3}_interface.h`` and
``include/interface/extension_interface.h``; the ``sb_handle`` wraps a CUDA
stream and every buffer is a device pointer (a CUDA ``torch.Tensor`` or a raw
integer address).  Each call forwards to the C ABI of ``libgbblas.so``
(``include/gbblas.h``); nothing here computes.

Errors mirror portBLAS's: ``std::invalid_argument`` becomes
``InvalidArgument`` (a ``ValueError``) and ``blas::unsupported_exception``
becomes ``UnsupportedException``; CUDA failures raise ``GbblasError`` instead
of being swallowed.

Async vs sync BLAS-1: as in portBLAS, passing a device result buffer ``rs``
enqueues the reduction and returns an event list; omitting it blocks and
returns the scalar (``blas1_interface.h:903-1000``).  The async forms
overwrite ``rs`` (portBLAS adds into it; its tests zero it first).
"""
from __future__ import annotations

import ctypes as C
import enum

from . import _lib


class GbblasError(RuntimeError):
    """A CUDA / runtime failure reported by libgbblas."""


class InvalidArgument(ValueError):
    """portBLAS throws std::invalid_argument (gemm_interface.hpp:144-166)."""


class UnsupportedException(NotImplementedError):
    """portBLAS blas::unsupported_exception (include/blas_meta.h:225-235)."""


_STATUS = {1: InvalidArgument, 2: UnsupportedException, 3: GbblasError, 4: GbblasError, 5: MemoryError,
           6: GbblasError}


def _check(status: int) -> None:
    if status == 0:
        return
    L = _lib.load()
    msg = (L.gbblas_last_error() or b"").decode() or L.gbblas_status_string(status).decode()
    raise _STATUS.get(status, GbblasError)(msg)


class gemm_batch_type_t(enum.IntEnum):
    strided = 0
    interleaved = 1


class reduction_dim_t(enum.IntEnum):
    inner = 0
    outer = 1


class sgemm_mode_t(enum.IntEnum):
    auto = 0
    fp32_simt = 1
    split_bf16x3 = 2
    split_bf16x6 = 3


# operator tags of blas::extension::_reduction<operator_t, element_t>
class AddOperator: code = 0
class ProductOperator: code = 1
class MaxOperator: code = 2
class MinOperator: code = 3
class AbsoluteAddOperator: code = 4
class MeanOperator: code = 5


def _ptr(x):
    """Device address of a CUDA tensor or an integer address."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise InvalidArgument("buffers must live in device memory (got a host tensor)")
        return x.data_ptr()
    raise TypeError(f"expected a CUDA tensor or a device address, got {type(x).__name__}")


def _prefix(x, dtype=None) -> str:
    """'s' or 'd' from the tensor dtype (or an explicit dtype string)."""
    if dtype is not None:
        name = str(dtype)
    elif hasattr(x, "dtype"):
        name = str(x.dtype)
    else:
        raise TypeError("raw device addresses need dtype='float32' or 'float64'")
    if "float32" in name:
        return "s"
    if "float64" in name:
        return "d"
    raise UnsupportedException(f"element type {name} is not supported on this path")


def _ch(t) -> bytes:
    if isinstance(t, bytes):
        return t[:1]
    return str(t).encode()[:1]


class SB_Handle:
    """blas::SB_Handle over a CUDA stream (include/sb_handle/portblas_handle.h:46-200).

    ``stream`` may be a ``torch.cuda.Stream``, a raw ``cudaStream_t`` value or
    None for the current torch stream (or the legacy default stream)."""

    def __init__(self, stream=None):
        self._L = _lib.load()
        self.stream = stream
        raw = self._raw_stream(stream)
        h = C.c_void_p()
        _check(self._L.gbblas_handle_create(raw, C.byref(h)))
        self._h = h

    @staticmethod
    def _raw_stream(stream):
        if stream is None:
            try:
                import torch
                return torch.cuda.current_stream().cuda_stream
            except Exception:
                return None
        if isinstance(stream, int):
            return stream
        return stream.cuda_stream

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream) -> None:
        self.stream = stream
        _check(self._L.gbblas_set_stream(self._h, self._raw_stream(stream)))

    def get_stream(self) -> int:
        s = C.c_void_p()
        _check(self._L.gbblas_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def wait(self, events=None) -> None:
        """SB_Handle::wait: blocks until the handle's stream is idle."""
        _check(self._L.gbblas_wait(self._h))

    def temp_bytes(self) -> int:
        n = C.c_size_t()
        _check(self._L.gbblas_temp_bytes(self._h, C.byref(n)))
        return n.value

    def check_device_error(self) -> None:
        _check(self._L.gbblas_check_device_error(self._h))

    def set_sgemm_mode(self, mode) -> None:
        _check(self._L.gbblas_set_sgemm_mode(self._h, int(mode)))

    def get_sgemm_mode(self) -> int:
        m = C.c_int()
        _check(self._L.gbblas_get_sgemm_mode(self._h, C.byref(m)))
        return m.value

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.gbblas_handle_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _call(name: str, *args):
    _check(getattr(_lib.load(), name)(*args))
    return []  # event_t: work is ordered on the handle's stream


def launch_count() -> int:
    return int(_lib.load().gbblas_launch_count())


# ------------------------------------------------------------- BLAS-3 --
def _gemm(sb_handle, transa, transb, M, N, K, alpha, a, lda, b, ldb, beta, c, ldc, dependencies=None, dtype=None):
    """blas::_gemm (include/interface/blas3_interface.h:86-95)."""
    p = _prefix(c, dtype)
    return _call(f"gbblas_{p}gemm", sb_handle.handle, _ch(transa), _ch(transb), M, N, K, alpha, _ptr(a), lda,
                 _ptr(b), ldb, beta, _ptr(c), ldc)


def _gemm_batched(sb_handle, transa, transb, M, N, K, alpha, a, lda, b, ldb, beta, c, ldc, batch_size,
                  batch_type=gemm_batch_type_t.strided, dependencies=None, dtype=None):
    """blas::_gemm_batched (include/interface/blas3_interface.h:97-109)."""
    p = _prefix(c, dtype)
    return _call(f"gbblas_{p}gemm_batched", sb_handle.handle, _ch(transa), _ch(transb), M, N, K, alpha, _ptr(a),
                 lda, _ptr(b), ldb, beta, _ptr(c), ldc, batch_size, int(batch_type))


def _gemm_strided_batched(sb_handle, transa, transb, M, N, K, alpha, a, lda, stridea, b, ldb, strideb, beta, c,
                          ldc, stridec, batch_size, dependencies=None, dtype=None):
    """blas::_gemm_strided_batched (include/interface/blas3_interface.h:111-123)."""
    p = _prefix(c, dtype)
    return _call(f"gbblas_{p}gemm_strided_batched", sb_handle.handle, _ch(transa), _ch(transb), M, N, K, alpha,
                 _ptr(a), lda, stridea, _ptr(b), ldb, strideb, beta, _ptr(c), ldc, stridec, batch_size)


# ------------------------------------------------------------- BLAS-2 --
def _gemv(sb_handle, trans, M, N, alpha, a, lda, x, incx, beta, y, incy, dependencies=None, dtype=None):
    """blas::_gemv (include/interface/blas2_interface.h:632-655)."""
    p = _prefix(y, dtype)
    return _call(f"gbblas_{p}gemv", sb_handle.handle, _ch(trans), M, N, alpha, _ptr(a), lda, _ptr(x), incx, beta,
                 _ptr(y), incy)


# ------------------------------------------------------------- BLAS-1 --
def _scalar_out(p: str):
    return C.c_float() if p == "s" else C.c_double()


def _asum(sb_handle, N, x, incx, rs=None, dependencies=None, dtype=None):
    """blas::_asum: async with ``rs`` (blas1_interface.h:631-637), sync without (:979-984)."""
    p = _prefix(x, dtype)
    if rs is not None:
        return _call(f"gbblas_{p}asum", sb_handle.handle, N, _ptr(x), incx, _ptr(rs))
    out = _scalar_out(p)
    _call(f"gbblas_{p}asum_sync", sb_handle.handle, N, _ptr(x), incx, C.addressof(out))
    return out.value


def _nrm2(sb_handle, N, x, incx, rs=None, dependencies=None, dtype=None):
    """blas::_nrm2: async with ``rs`` (blas1_interface.h:712-718), sync without (:995-1000)."""
    p = _prefix(x, dtype)
    if rs is not None:
        return _call(f"gbblas_{p}nrm2", sb_handle.handle, N, _ptr(x), incx, _ptr(rs))
    out = _scalar_out(p)
    _call(f"gbblas_{p}nrm2_sync", sb_handle.handle, N, _ptr(x), incx, C.addressof(out))
    return out.value


def _dot(sb_handle, N, x, incx, y, incy, rs=None, dependencies=None, dtype=None):
    """blas::_dot: async with ``rs`` (blas1_interface.h:582-588), sync without (:903-909)."""
    p = _prefix(x, dtype)
    if rs is not None:
        return _call(f"gbblas_{p}dot", sb_handle.handle, N, _ptr(x), incx, _ptr(y), incy, _ptr(rs))
    out = _scalar_out(p)
    _call(f"gbblas_{p}dot_sync", sb_handle.handle, N, _ptr(x), incx, _ptr(y), incy, C.addressof(out))
    return out.value


def _iamax(sb_handle, N, x, incx, rs=None, dependencies=None, dtype=None):
    """blas::_iamax: async with an int32 ``rs`` (blas1_interface.h:646-655), sync without (:949-957)."""
    p = _prefix(x, dtype)
    if rs is not None:
        return _call(f"gbblas_i{p}amax", sb_handle.handle, N, _ptr(x), incx, _ptr(rs))
    out = C.c_int32()
    _call(f"gbblas_i{p}amax_sync", sb_handle.handle, N, _ptr(x), incx, C.addressof(out))
    return out.value


def _iamin(sb_handle, N, x, incx, rs=None, dependencies=None, dtype=None):
    """blas::_iamin: async with an int32 ``rs`` (blas1_interface.h:657-666), sync without (:960-968)."""
    p = _prefix(x, dtype)
    if rs is not None:
        return _call(f"gbblas_i{p}amin", sb_handle.handle, N, _ptr(x), incx, _ptr(rs))
    out = C.c_int32()
    _call(f"gbblas_i{p}amin_sync", sb_handle.handle, N, _ptr(x), incx, C.addressof(out))
    return out.value


def _scal(sb_handle, N, alpha, x, incx, dependencies=None, dtype=None):
    """blas::_scal (include/interface/blas1_interface.h:697-701)."""
    p = _prefix(x, dtype)
    return _call(f"gbblas_{p}scal", sb_handle.handle, N, alpha, _ptr(x), incx)


def _axpy(sb_handle, N, alpha, x, incx, y, incy, dependencies=None, dtype=None):
    """blas::_axpy (include/interface/blas1_interface.h:536-541)."""
    p = _prefix(y, dtype)
    return _call(f"gbblas_{p}axpy", sb_handle.handle, N, alpha, _ptr(x), incx, _ptr(y), incy)


def _copy(sb_handle, N, x, incx, y, incy, dependencies=None, dtype=None):
    """blas::_copy (include/interface/blas1_interface.h:556-560)."""
    p = _prefix(y, dtype)
    return _call(f"gbblas_{p}copy", sb_handle.handle, N, _ptr(x), incx, _ptr(y), incy)


def _sdsdot(sb_handle, N, sb, x, incx, y, incy, rs=None, dependencies=None):
    """blas::_sdsdot: async with ``rs`` (blas1_interface.h:615-620), sync without."""
    if rs is not None:
        return _call("gbblas_sdsdot", sb_handle.handle, N, sb, _ptr(x), incx, _ptr(y), incy, _ptr(rs))
    import torch
    r = torch.empty(1, dtype=torch.float32, device="cuda")
    _call("gbblas_sdsdot", sb_handle.handle, N, sb, _ptr(x), incx, _ptr(y), incy, _ptr(r))
    return float(r.item())


def _symm(sb_handle, side, uplo, M, N, alpha, a, lda, b, ldb, beta, c, ldc, dependencies=None, dtype=None):
    """blas::_symm (include/interface/blas3_interface.h:135-145)."""
    p = _prefix(c, dtype)
    return _call(f"gbblas_{p}symm", sb_handle.handle, _ch(side), _ch(uplo), M, N, alpha, _ptr(a), lda, _ptr(b), ldb,
                 beta, _ptr(c), ldc)


# ---------------------------------------------------------- extension --
class extension:
    """blas::extension namespace."""

    @staticmethod
    def _omatcopy(sb_handle, trans, m, n, alpha, in_memory, ld_in, out_memory, ld_out, dependencies=None,
                  dtype=None):
        """blas::extension::_omatcopy (include/interface/extension_interface.h:188-198)."""
        p = _prefix(in_memory, dtype)
        return _call(f"gbblas_{p}omatcopy", sb_handle.handle, _ch(trans), m, n, alpha, _ptr(in_memory), ld_in,
                     _ptr(out_memory), ld_out)

    @staticmethod
    def _transpose(sb_handle, m, n, A, ld_a, B=None, ld_b=None, dependencies=None, dtype=None):
        """blas::extension::_transpose: out of place (A -> B, ld_b) or, with
        B omitted and ld_b the output leading dimension, in place
        (include/interface/extension_interface.h:405-452)."""
        p = _prefix(A, dtype)
        if B is None or isinstance(B, int) and ld_b is None:
            ld_out = B if ld_b is None else ld_b
            return _call(f"gbblas_{p}transpose_inplace", sb_handle.handle, m, n, _ptr(A), ld_a, ld_out)
        return _call(f"gbblas_{p}transpose", sb_handle.handle, m, n, _ptr(A), ld_a, _ptr(B), ld_b)

    @staticmethod
    def _reduction(operator_t, sb_handle, buffer_in, ld, buffer_out, rows, cols, reduction_dim,
                   dependencies=None, dtype=None):
        """blas::extension::_reduction<operator_t, element_t>
        (include/interface/extension_interface.h:453-462)."""
        p = _prefix(buffer_in, dtype)
        return _call(f"gbblas_{p}reduction", sb_handle.handle, int(operator_t.code), int(reduction_dim),
                     _ptr(buffer_in), ld, _ptr(buffer_out), rows, cols)


# --------------------------------------------------------- grouped GEMM --
_DTYPE_CODES = {"float32": 0, "bfloat16": 1, "float64": 2, "torch.float32": 0, "torch.bfloat16": 1,
                "torch.float64": 2}


def _dtype_code(dtype) -> int:
    try:
        return _DTYPE_CODES[str(dtype)]
    except KeyError:
        raise UnsupportedException(f"grouped GEMM: element type {dtype} is not supported") from None


def _grouped_arrays(problems):
    cnt = len(problems)
    I64 = C.c_int64 * cnt
    F32 = C.c_float * cnt
    VP = C.c_void_p * cnt
    ta = C.create_string_buffer(bytes(_ch(p["transa"])[0] for p in problems), cnt)
    tb = C.create_string_buffer(bytes(_ch(p["transb"])[0] for p in problems), cnt)
    arrs = dict(
        m=I64(*[p["m"] for p in problems]), n=I64(*[p["n"] for p in problems]), k=I64(*[p["k"] for p in problems]),
        alpha=F32(*[p["alpha"] for p in problems]), beta=F32(*[p["beta"] for p in problems]),
        a=VP(*[_ptr(p["a"]) for p in problems]), b=VP(*[_ptr(p["b"]) for p in problems]),
        c=VP(*[_ptr(p["c"]) for p in problems]), lda=I64(*[p["lda"] for p in problems]),
        ldb=I64(*[p["ldb"] for p in problems]), ldc=I64(*[p["ldc"] for p in problems]))
    A = lambda x: C.addressof(x)
    keep = (ta, tb, arrs)
    args = (cnt, A(ta), A(tb), A(arrs["m"]), A(arrs["n"]), A(arrs["k"]), A(arrs["alpha"]), A(arrs["a"]),
            A(arrs["lda"]), A(arrs["b"]), A(arrs["ldb"]), A(arrs["beta"]), A(arrs["c"]), A(arrs["ldc"]))
    return args, keep


def _gemm_grouped(sb_handle, problems, dtype="float32"):
    """Grouped GEMM over uneven problems (no portBLAS counterpart), one
    persistent launch.  ``problems`` is a list of dicts with keys transa,
    transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc (a/b/c CUDA tensors or
    addresses); A and B are ``dtype`` (float32 or bfloat16), C is float32."""
    args, keep = _grouped_arrays(problems)
    return _call("gbblas_gemm_grouped", sb_handle.handle, _dtype_code(dtype), *args)


def sgemm_split_route(m, n, k, batch=1, mode=sgemm_mode_t.split_bf16x3, sm_count=152):
    """Host-side tile choice of the fixed split-BF16 modes for an m x n x k
    GEMM of ``batch`` matrices on a GPU with ``sm_count`` SMs:
    (tile_m, tile_n, k_slices); tile_m 256 is a CTA pair sharing one tile."""
    L = _lib.load()
    tm, tn, ks = C.c_int(), C.c_int(), C.c_int()
    _check(L.gbblas_sgemm_split_route(int(m), int(n), int(k), int(batch), int(mode), int(sm_count), C.byref(tm),
                                      C.byref(tn), C.byref(ks)))
    return tm.value, tn.value, ks.value


def grouped_schedule(problems, dtype="float32", sm_count=152):
    """Host-side tile schedule of a tcgen05 grouped GEMM over ``problems``
    (dicts with transa, transb, m, n, k, alpha) on a GPU with ``sm_count``
    SMs: (tiles handed out, K slices per problem; 0 for an empty problem)."""
    L = _lib.load()
    cnt = len(problems)
    I64 = C.c_int64 * max(cnt, 1)
    F32 = C.c_float * max(cnt, 1)
    ta = C.create_string_buffer(bytes(_ch(p["transa"])[0] for p in problems), max(cnt, 1))
    tb = C.create_string_buffer(bytes(_ch(p["transb"])[0] for p in problems), max(cnt, 1))
    m, n, k = (I64(*[p[key] for p in problems]) for key in ("m", "n", "k"))
    alpha = F32(*[p["alpha"] for p in problems])
    tiles = C.c_int64()
    splits = (C.c_int * max(cnt, 1))()
    _check(L.gbblas_grouped_schedule(_dtype_code(dtype), cnt, C.addressof(ta), C.addressof(tb), C.addressof(m),
                                     C.addressof(n), C.addressof(k), C.addressof(alpha), int(sm_count),
                                     C.byref(tiles), C.addressof(splits)))
    return tiles.value, list(splits)[:cnt]


class GroupedPlan:
    """A reusable grouped GEMM replayed from a CUDA graph
    (gbblas_grouped_plan_create / _run / _destroy)."""

    def __init__(self, sb_handle, problems, dtype="float32"):
        self._L = _lib.load()
        self.sb = sb_handle
        args, self._keep = _grouped_arrays(problems)
        p = C.c_void_p()
        _check(self._L.gbblas_grouped_plan_create(sb_handle.handle, _dtype_code(dtype), *args, C.byref(p)))
        self._p = p

    def run(self):
        _check(self._L.gbblas_grouped_plan_run(self.sb.handle, self._p))
        return []

    def info(self):
        """(tiles handed out, largest number of K slices of any problem)."""
        tiles, splits = C.c_int64(), C.c_int()
        _check(self._L.gbblas_grouped_plan_info(self._p, C.byref(tiles), C.byref(splits)))
        return tiles.value, splits.value

    def close(self):
        if getattr(self, "_p", None) is not None and self._p.value:
            self._L.gbblas_grouped_plan_destroy(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
