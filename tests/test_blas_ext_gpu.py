"""The element-wise BLAS-1 neighbours (_scal, _axpy, _copy, _sdsdot), the
matrix copy/transpose extensions and _symm against the oracle, through the
C ABI, with strided and negative increments and ragged sizes."""
import numpy as np
import pytest

import oracle
from tests.util import rng, to_dev, to_host, assert_almost_equal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 11, 1002, 1 << 20])
@pytest.mark.parametrize("incx,incy", [(1, 1), (3, 2), (-2, 1), (1, -3)])
def test_axpy_copy_scal(sb, torch_cuda, n, incx, incy):
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(n + incx * 7 + incy)
    x = g.uniform(-2, 5, n * abs(incx)).astype(np.float32)
    y = g.uniform(-2, 5, n * abs(incy)).astype(np.float32)
    yd = to_dev(y, torch)
    blas._axpy(sb, n, 1.5, to_dev(x, torch), incx, yd, incy)
    assert_almost_equal(to_host(yd), oracle.axpy(n, 1.5, x, incx, y, incy))
    yd = to_dev(y, torch)
    blas._copy(sb, n, to_dev(x, torch), incx, yd, incy)
    np.testing.assert_array_equal(to_host(yd), oracle.copy(n, x, incx, y, incy).astype(np.float32))
    xd = to_dev(x, torch)
    blas._scal(sb, n, -0.75, xd, incx)
    np.testing.assert_array_equal(to_host(xd), oracle.scal(n, -0.75, x, incx).astype(np.float32))
    xn = x.copy()
    xn[::max(1, abs(incx))][:3] = np.nan
    xd = to_dev(xn, torch)
    blas._scal(sb, n, 0.0, xd, incx)  # alpha == 0 writes zeros, NaN included
    np.testing.assert_array_equal(to_host(xd), oracle.scal(n, 0.0, xn, incx).astype(np.float32))


@pytest.mark.parametrize("n", [0, 11, 1002, 1002400])
def test_sdsdot(sb, torch_cuda, n):
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(n + 3)
    x = g.uniform(-2, 5, max(n, 1)).astype(np.float32)
    y = g.uniform(-2, 5, max(n, 1)).astype(np.float32)
    got = blas._sdsdot(sb, n, 0.5, to_dev(x, torch), 1, to_dev(y, torch), 1)
    assert_almost_equal(got, oracle.sdsdot(n, 0.5, x, 1, y, 1))


@pytest.mark.parametrize("trans", ["n", "t"])
@pytest.mark.parametrize("m,n,ld_in_add,ld_out_add", [(1, 1, 0, 0), (33, 65, 3, 1), (1000, 513, 0, 7)])
def test_omatcopy(sb, torch_cuda, trans, m, n, ld_in_add, ld_out_add):
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(m * n)
    ld_in = m + ld_in_add
    ld_out = (m if trans == "n" else n) + ld_out_add
    a = g.uniform(-2, 5, ld_in * n).astype(np.float32)
    out = g.uniform(-2, 5, ld_out * (n if trans == "n" else m)).astype(np.float32)
    od = to_dev(out, torch)
    blas.extension._omatcopy(sb, trans, m, n, 2.0, to_dev(a, torch), ld_in, od, ld_out)
    np.testing.assert_array_equal(to_host(od), oracle.omatcopy(trans, m, n, 2.0, a, ld_in, out, ld_out).astype(np.float32))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_transpose_out_of_place_and_in_place(sb, torch_cuda, dtype):
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(5)
    m, n = 300, 77
    a = g.uniform(-2, 5, m * n).astype(dtype)
    ref = a.reshape(n, m).T.copy()  # m x n
    b = torch.zeros(n * m, device="cuda", dtype=torch.float32 if dtype == np.float32 else torch.float64)
    blas.extension._transpose(sb, m, n, to_dev(a, torch), m, b, n)
    np.testing.assert_array_equal(to_host(b).reshape(m, n).T, ref.T)
    ad = to_dev(a, torch)
    blas.extension._transpose(sb, m, n, ad, m, n)  # in place, ld_out = n
    np.testing.assert_array_equal(to_host(ad).reshape(m, n).T, ref.T)


@pytest.mark.parametrize("side", ["l", "r"])
@pytest.mark.parametrize("uplo", ["u", "l"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_symm(sb, torch_cuda, side, uplo, dtype):
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(17 + (side == "l") + 2 * (uplo == "u"))
    m, n = 67, 45
    na = m if side == "l" else n
    lda, ldb, ldc = na + 2, m + 1, m + 3
    a = g.uniform(-2, 5, lda * na).astype(dtype)
    b = g.uniform(-2, 5, ldb * n).astype(dtype)
    c = g.uniform(-2, 5, ldc * n).astype(dtype)
    ref = oracle.symm(side, uplo, m, n, 1.5, a, lda, b, ldb, 0.5, c, ldc)
    cd = to_dev(c, torch)
    blas._symm(sb, side, uplo, m, n, 1.5, to_dev(a, torch), lda, to_dev(b, torch), ldb, 0.5, cd, ldc)
    got = to_host(cd).reshape(n, ldc).T[:m]
    assert_almost_equal(got, ref, dtype=dtype)
    with pytest.raises(blas.InvalidArgument):
        blas._symm(sb, "x", uplo, m, n, 1.5, to_dev(a, torch), lda, to_dev(b, torch), ldb, 0.5, cd, ldc)
