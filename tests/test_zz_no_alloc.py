"""The allocation-free GEMV entry point (gbblas_sgemv_noalloc).

It exists for callers that cannot allocate device memory: hosts whose GPU
memory is owned by an allocator of their own, plug-in hosts that forbid
allocation once running, and loops that cannot take cudaMalloc's implicit
synchronisation.  Called here through the C ABI and compared with
gbblas_sgemv (the regular, allocating entry point) on two calls in a row, at
the GEMV tests' tolerance.  This file is collected last so that a run that
stops at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from tests.util import rng

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L(torch_cuda):
    from portblas_gb300 import _lib, build
    build.build()
    return _lib.load()


def _stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("trans", ["n", "t"])
@pytest.mark.parametrize("m,n,lda,incx,incy,beta", [(8192, 8192, 8192, 1, 1, 0.0), (1000, 700, 1002, 2, 3, 0.5),
                                                     (37, 5000, 40, 1, 1, 1.5)])
def test_noalloc_matches_sgemv_twice(L, torch_cuda, trans, m, n, lda, incx, incy, beta):
    torch = torch_cuda
    g = rng(m + n + lda)
    a = torch.from_numpy(g.uniform(-1, 1, lda * n).astype(np.float32)).cuda()
    xlen, ylen = (n, m) if trans == "n" else (m, n)
    h = C.c_void_p()
    assert L.gbblas_handle_create(_stream(torch), C.byref(h)) == 0
    try:
        for call in range(2):  # two calls in a row share the static scratch
            x = torch.from_numpy(g.uniform(-1, 1, xlen * incx).astype(np.float32)).cuda()
            y0 = torch.from_numpy(g.uniform(-1, 1, ylen * incy).astype(np.float32)).cuda()
            y_ref, y_new = y0.clone(), y0.clone()
            st = L.gbblas_sgemv(h, trans.encode(), m, n, 1.5, a.data_ptr(), lda, x.data_ptr(), incx, beta,
                                y_ref.data_ptr(), incy)
            assert st == 0, L.gbblas_last_error()
            st = L.gbblas_sgemv_noalloc(_stream(torch), trans.encode(), m, n, 1.5, a.data_ptr(), lda, x.data_ptr(),
                                        incx, beta, y_new.data_ptr(), incy)
            assert st == 0, L.gbblas_last_error()
            torch.cuda.synchronize()
            ref, got = y_ref.cpu().numpy(), y_new.cpu().numpy()
            np.testing.assert_allclose(got, ref, rtol=2e-5, atol=2e-5 * np.abs(ref).max(), err_msg=f"call {call}")
    finally:
        L.gbblas_handle_destroy(h)


def test_noalloc_rejects_scratch_beyond_maximum(L, torch_cuda):
    """A problem whose split partials exceed the fixed 1 MiB block is refused
    with INVALID_ARG before anything runs (the pointers are never touched)."""
    torch = torch_cuda
    buf = torch.zeros(64, device="cuda")
    p = buf.data_ptr()
    m, n = 1 << 23, 1 << 9  # transposed sweep: thousands of row chunks x 512 columns of partials, >> 1 MiB
    st = L.gbblas_sgemv_noalloc(_stream(torch), b"t", m, n, 1.0, p, m, p, 1, 0.0, p, 1)
    assert st == 1
    assert b"allocation-free maximum" in L.gbblas_last_error()
    torch.cuda.synchronize()


def test_noalloc_rejects_bad_arguments_before_enqueueing(L, torch_cuda):
    """Argument errors come back as INVALID_ARG, as from gbblas_sgemv."""
    torch = torch_cuda
    buf = torch.zeros(64, device="cuda")
    p = buf.data_ptr()
    assert L.gbblas_sgemv_noalloc(_stream(torch), b"n", -1, 4, 1.0, p, 4, p, 1, 0.0, p, 1) == 1
    assert L.gbblas_sgemv_noalloc(_stream(torch), b"n", 4, 4, 1.0, p, 4, p, 0, 0.0, p, 1) == 1
    assert L.gbblas_sgemv_noalloc(_stream(torch), b"n", 4, 4, 1.0, None, 4, p, 1, 0.0, p, 1) == 1
    torch.cuda.synchronize()
