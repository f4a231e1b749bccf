"""GPU parity of _gemv against the oracle through the C ABI, on portBLAS's
sweep (test/unittest/blas2/blas2_gemv_test.cpp:123-151) plus edge cases."""
import numpy as np
import pytest

import oracle
from tests.util import rng, to_dev, to_host, assert_almost_equal

pytestmark = pytest.mark.gpu


def _run(sb, torch, trans, m, n, alpha, beta, incx, incy, lda_mul=1, dtype=np.float32, seed=0, y_nan=False):
    from portblas_gb300 import blas
    g = rng(seed + m + n)
    lda = m * lda_mul
    a = g.uniform(-2, 5, lda * n).astype(dtype)
    xlen, ylen = (n, m) if trans in "nN" else (m, n)
    x = g.uniform(-2, 5, xlen * abs(incx)).astype(dtype)
    y = g.uniform(-2, 5, ylen * abs(incy)).astype(dtype)
    if y_nan:
        y[:] = np.nan
    ref = oracle.gemv(trans, m, n, alpha, a, lda, x, incx, beta, y, incy)
    yd = to_dev(y, torch)
    blas._gemv(sb, trans, m, n, alpha, to_dev(a, torch), lda, to_dev(x, torch), incx, beta, yd, incy)
    got = oracle.view(to_host(yd), ylen, incy)
    return got, ref


@pytest.mark.parametrize("trans", ["n", "t"])
@pytest.mark.parametrize("m,n", [(11, 14), (11, 1010), (1023, 14), (1023, 1010)])
@pytest.mark.parametrize("beta", [0.0, 1.5])
@pytest.mark.parametrize("incx,incy,lda_mul", [(2, 3, 2), (1, 1, 1), (-1, 2, 1)])
def test_gemv_sweep(sb, torch_cuda, trans, m, n, beta, incx, incy, lda_mul):
    got, ref = _run(sb, torch_cuda, trans, m, n, 1.5, beta, incx, incy, lda_mul)
    assert_almost_equal(got, ref)
    np.testing.assert_allclose(got, ref, rtol=2e-5, atol=2e-5 * np.abs(ref).max())


@pytest.mark.parametrize("trans", ["n", "t"])
def test_gemv_beta0_ignores_nan_y(sb, torch_cuda, trans):
    got, ref = _run(sb, torch_cuda, trans, 37, 29, 1.0, 0.0, 1, 1, y_nan=True)
    assert np.all(np.isfinite(got))
    assert_almost_equal(got, ref)


@pytest.mark.parametrize("trans", ["n", "t"])
@pytest.mark.parametrize("m,n", [(1, 1), (1, 3000), (3000, 1), (5, 0), (0, 5), (257, 131)])
def test_gemv_edges(sb, torch_cuda, trans, m, n):
    got, ref = _run(sb, torch_cuda, trans, m, n, 0.75, 0.25, 1, 1)
    assert_almost_equal(got, ref)


@pytest.mark.parametrize("trans", ["n", "t"])
def test_gemv_double(sb, torch_cuda, trans):
    got, ref = _run(sb, torch_cuda, trans, 513, 257, 1.5, 0.5, 1, 2, dtype=np.float64)
    assert_almost_equal(got, ref, dtype=np.float64)


@pytest.mark.parametrize("trans", ["n", "t"])
def test_gemv_full_size_linearity(sb, torch_cuda, trans):
    """8192 x 8192 (the benchmark size): y(A, x1 + x2) == y(A, x1) + y(A, x2)
    to FP32 rounding, and a sampled row set against the oracle."""
    torch = torch_cuda
    from portblas_gb300 import blas
    m = n = 8192
    gen = torch.Generator(device="cuda").manual_seed(5)
    a = torch.rand(m * n, device="cuda", generator=gen) * 2 - 1
    x1 = torch.rand(8192, device="cuda", generator=gen) * 2 - 1
    x2 = torch.rand(8192, device="cuda", generator=gen) * 2 - 1
    ys = [torch.empty(8192, device="cuda") for _ in range(3)]
    for y, x in zip(ys, (x1, x2, x1 + x2)):
        blas._gemv(sb, trans, m, n, 1.0, a, m, x, 1, 0.0, y, 1)
    lin = (ys[0] + ys[1] - ys[2]).abs().max().item()
    assert lin <= 1e-3
    A = a.view(n, m).T.double()
    ref = (A @ x1.double()) if trans == "n" else (A.T @ x1.double())
    err = (ys[0].double() - ref).abs().max().item()
    assert err <= 2e-5 * ref.abs().max().item() * 8


@pytest.mark.parametrize("trans", ["n", "t"])
@pytest.mark.parametrize("m,n,lda", [(1000, 700, 1000), (4100, 300, 4104), (520, 1030, 520), (8192, 257, 8192),
                                     (257, 5000, 260), (30000, 2048, 30000)])
@pytest.mark.parametrize("beta", [0.0, 0.5])
def test_gemv_tma_stream_path(sb, torch_cuda, trans, m, n, lda, beta):
    """Shapes whose lda satisfies the tensor-map rules take the TMA-fed sweeps:
    ragged row/column tiles, split combines, strided x/y.  30000 x 2048 'n':
    235 row tiles, fewer than two per SM in one wave, so the column split
    comes from the wave cost (3 splits of 22, 22 and 20 tiles)."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(m + n + lda)
    a = g.uniform(-1, 1, lda * n).astype(np.float32)
    xlen, ylen = (n, m) if trans == "n" else (m, n)
    x = g.uniform(-1, 1, xlen * 2).astype(np.float32)
    y = g.uniform(-1, 1, ylen * 3).astype(np.float32)
    ref = oracle.gemv(trans, m, n, 1.25, a, lda, x, 2, beta, y, 3)
    yd = to_dev(y, torch)
    blas._gemv(sb, trans, m, n, 1.25, to_dev(a, torch), lda, to_dev(x, torch), 2, beta, yd, 3)
    got = oracle.view(to_host(yd), ylen, 3)
    assert_almost_equal(got, ref)
    np.testing.assert_allclose(got, ref, rtol=2e-5, atol=2e-5 * np.abs(ref).max())
    # entries of y between the strided elements are untouched
    yo = to_host(yd)
    mask = np.ones(len(y), bool)
    mask[: ylen * 3: 3] = False
    np.testing.assert_array_equal(yo[mask], y[mask])


@pytest.mark.parametrize("m,n,lda", [(1001, 2500, 1004), (3, 3000, 4), (4096, 9728, 4096), (130, 1300, 132),
                                     (5, 1216, 8), (8193, 4865, 8196)])
@pytest.mark.parametrize("beta,incy", [(0.0, 1), (0.5, 3)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_gemv_t_warp_per_column_path(sb, torch_cuda, m, n, lda, beta, incy, dtype):
    """Transposed GEMV over many columns with contiguous x and 16-byte-aligned
    columns (a CTA per group of columns, its warps over equal row ranges):
    ragged column lengths (vector part plus scalar tail, or the tail alone,
    fewer vectors than warps), one to sixteen columns per CTA, strided y;
    every entry against the oracle and y's gaps untouched."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(m + n + lda + incy)
    a = g.uniform(-1, 1, lda * n).astype(dtype)
    x = g.uniform(-1, 1, m).astype(dtype)
    y = g.uniform(-1, 1, n * incy).astype(dtype)
    ref = oracle.gemv("t", m, n, 1.25, a, lda, x, 1, beta, y, incy)
    yd = to_dev(y, torch)
    blas._gemv(sb, "t", m, n, 1.25, to_dev(a, torch), lda, to_dev(x, torch), 1, beta, yd, incy)
    got = oracle.view(to_host(yd), n, incy)
    tol = 2e-5 if dtype == np.float32 else 1e-12
    np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * np.abs(ref).max())
    if incy > 1:
        yo = to_host(yd)
        mask = np.ones(len(y), bool)
        mask[::incy] = False
        np.testing.assert_array_equal(yo[mask], y[mask])


@pytest.mark.parametrize("m,n,lda,off", [(1001, 2500, 1001, 0), (1003, 3001, 1005, 1), (2, 2000, 3, 3),
                                         (4097, 1500, 4099, 2)])
def test_gemv_t_warp_per_column_misaligned(sb, torch_cuda, m, n, lda, off):
    """Transposed GEMV with columns that start off a 16-byte boundary (odd lda,
    A and x at an element offset): each column's head read element-wise, the
    rest as 16-byte vectors, against the oracle."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(m + n + lda + off)
    a = g.uniform(-1, 1, lda * n + off).astype(np.float32)
    x = g.uniform(-1, 1, m + off).astype(np.float32)
    y = g.uniform(-1, 1, n).astype(np.float32)
    ref = oracle.gemv("t", m, n, 0.75, a[off:], lda, x[off:], 1, 0.5, y, 1)
    ad, xd, yd = to_dev(a, torch), to_dev(x, torch), to_dev(y, torch)
    blas._gemv(sb, "t", m, n, 0.75, ad[off:], lda, xd[off:], 1, 0.5, yd, 1)
    np.testing.assert_allclose(to_host(yd), ref, rtol=2e-5, atol=2e-5 * np.abs(ref).max())


@pytest.mark.parametrize("trans", ["n", "t"])
@pytest.mark.parametrize("m,n,lda,incx,incy", [(8, 1 << 22, 8, 1, 1), (3, 70001, 3, 1, 1), (32, 20000, 32, 2, 3),
                                               (17, 5003, 20, -1, 2), (1, 9000, 1, 1, 1), (5, 64, 7, 3, 1),
                                               (32, 1, 32, 1, 1), (12, 0, 12, 1, 1), (64, 1 << 18, 64, 1, 1),
                                               (33, 9001, 36, 1, 2), (48, 3000, 49, -2, 1), (100, 20001, 100, 1, 1),
                                               (128, 3001, 130, 1, 3), (65, 777, 65, -1, 1)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_gemv_narrow_rows(sb, torch_cuda, trans, m, n, lda, incx, incy, dtype):
    """Short, wide A (up to 128 FP32 / 64 FP64 rows; FP64 rows beyond take
    the general sweeps): 'n' runs rows_narrow (several columns per warp load,
    the CTAs' partials folded by the last CTA), 't' cols_thread (up to 32
    rows) or cols_lanes (a few lanes per column, shuffle-folded); packed,
    padded and odd leading dimensions, strided and reversed x, strided y, no
    columns at all."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(m + n + lda + int(dtype == np.float64))
    a = g.uniform(-1, 1, max(lda * n, 1)).astype(dtype)
    xlen, ylen = (n, m) if trans == "n" else (m, n)
    if ylen == 0:
        pytest.skip("no output")
    x = g.uniform(-1, 1, max(xlen * abs(incx), 1)).astype(dtype)
    y = g.uniform(-1, 1, ylen * incy).astype(dtype)
    ref = oracle.gemv(trans, m, n, 0.75, a, lda, x, incx, 0.5, y, incy)
    yd = to_dev(y, torch)
    blas._gemv(sb, trans, m, n, 0.75, to_dev(a, torch), lda, to_dev(x, torch), incx, 0.5, yd, incy)
    out = to_host(yd)
    got = oracle.view(out, ylen, incy)
    # error against the FP64 oracle, normalised by |alpha| |op(A)| |x| + |beta| |y|
    A2 = a[:lda * n].reshape(n, lda)[:, :m].astype(np.float64).T
    xv = np.abs(oracle.view(x, xlen, incx).astype(np.float64))
    scale = 0.75 * (np.abs(A2) @ xv if trans == "n" else np.abs(A2).T @ xv)
    scale = scale + 0.5 * np.abs(oracle.view(y, ylen, incy).astype(np.float64))
    assert (np.abs(got - ref) / scale).max() <= 256 * np.finfo(dtype).eps
    mask = np.ones(len(y), bool)
    mask[: ylen * incy: incy] = False
    np.testing.assert_array_equal(out[mask], y[mask])
    sb.check_device_error()


@pytest.mark.parametrize("trans", ["n", "t"])
@pytest.mark.parametrize("m,n,lda,incx,incy", [(20000, 8, 20000, 1, 1), (50001, 3, 50004, -1, 2),
                                               (30000, 32, 30001, 2, 1), (1 << 20, 17, 1 << 20, 1, 3)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_gemv_tall_narrow(sb, torch_cuda, trans, m, n, lda, incx, incy, dtype):
    """Tall, narrow A (at most 32 columns, rows beyond 64 per SM): 'n' runs
    rows_tall (a warp per 32 x RPT rows over every column); aligned and
    unaligned leading dimensions, ragged last rows, strided and reversed x,
    strided y; against the FP64 oracle, |A||x|-normalised."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(m + n + lda + int(dtype == np.float64))
    a = g.uniform(-1, 1, lda * n).astype(dtype)
    xlen, ylen = (n, m) if trans == "n" else (m, n)
    x = g.uniform(-1, 1, xlen * abs(incx)).astype(dtype)
    y = g.uniform(-1, 1, ylen * incy).astype(dtype)
    ref = oracle.gemv(trans, m, n, 0.75, a, lda, x, incx, 0.5, y, incy)
    yd = to_dev(y, torch)
    blas._gemv(sb, trans, m, n, 0.75, to_dev(a, torch), lda, to_dev(x, torch), incx, 0.5, yd, incy)
    out = to_host(yd)
    got = oracle.view(out, ylen, incy)
    A2 = a.reshape(n, lda)[:, :m].astype(np.float64).T
    xv = np.abs(oracle.view(x, xlen, incx).astype(np.float64))
    scale = 0.75 * (np.abs(A2) @ xv if trans == "n" else np.abs(A2).T @ xv)
    scale = scale + 0.5 * np.abs(oracle.view(y, ylen, incy).astype(np.float64))
    assert (np.abs(got - ref) / scale).max() <= 256 * np.finfo(dtype).eps
    mask = np.ones(len(y), bool)
    mask[: ylen * incy: incy] = False
    np.testing.assert_array_equal(out[mask], y[mask])
    sb.check_device_error()
