"""The CPU oracle pinned against portBLAS's known-answer tests and examples
(tests/golden/kat.json) and cross-checked against the CBLAS its tests link."""
import json
import os

import numpy as np
import pytest

import oracle
from tests.util import rng, assert_almost_equal

KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kat.json")))
FLT_MAX = float(np.finfo(np.float32).max)


def iaminmax_input(case):
    size, inc = case["n"], case["incx"]
    length = size * abs(inc)
    if case["mode"] == "limit":
        buf = np.full(length, case["fill"], dtype=np.float32)
    elif case["mode"] == "incrementing":
        buf = np.arange(length, dtype=np.float32)
    else:
        buf = (length - 1 - np.arange(length)).astype(np.float32)
    return buf


@pytest.mark.parametrize("case", KAT["iaminmax"], ids=lambda c: f"{c['op']}-{c['mode']}-{c['n']}-{c['incx']}")
def test_oracle_iaminmax_kat(case):
    x = iaminmax_input(case)
    fn = oracle.iamax if case["op"] == "iamax" else oracle.iamin
    assert fn(case["n"], x, case["incx"]) == case["expected"]


@pytest.mark.parametrize("case", KAT["reduction"], ids=lambda c: f"{c['op']}-{c['dim']}-ld{c['ld']}")
def test_oracle_reduction_kat(case):
    out = oracle.reduction(case["op"], case["dim"], np.array(case["data"]), case["ld"], case["rows"], case["cols"])
    np.testing.assert_array_equal(out, np.array(case["expected"]))


@pytest.mark.parametrize("case", KAT["gemm"], ids=lambda c: f"{c['ta']}{c['tb']}-a{c['alpha']}-b{c['beta']}-nan{c['c_nan']}")
def test_oracle_gemm_kat(case):
    c = np.array(case["c"], dtype=np.float64)
    if case["c_nan"]:
        c[:] = np.nan
    ta, tb = case["ta"].lower() != "n", case["tb"].lower() != "n"
    out = oracle.gemm(ta, tb, case["m"], case["n"], case["k"], case["alpha"], case["a"], case["lda"], case["b"],
                      case["ldb"], case["beta"], c, case["ldc"])
    np.testing.assert_array_equal(out.ravel(order="F"), np.array(case["expected"]))


@pytest.mark.parametrize("case", KAT["blas1"], ids=lambda c: f"{c['op']}-{c['n']}-{c['incx']}")
def test_oracle_blas1_kat(case):
    x = np.array(case["x"], dtype=np.float64)
    op = case["op"]
    if op == "asum":
        got = oracle.asum(case["n"], x, case["incx"])
    elif op == "nrm2":
        got = oracle.nrm2(case["n"], x, case["incx"])
    elif op == "dot":
        got = oracle.dot(case["n"], x, case["incx"], np.array(case["y"]), case["incy"])
    elif op == "iamax":
        got = oracle.iamax(case["n"], x, case["incx"])
    else:
        got = oracle.iamin(case["n"], x, case["incx"])
    assert got == pytest.approx(case["expected"], rel=1e-15)


def test_oracle_iamax_nan_and_empty():
    # NaN never wins; n == 0 leaves the initial tuple's index (INT_MAX)
    x = np.array([np.nan, 1.0, -3.0, np.nan, 3.0])
    assert oracle.iamax(5, x, 1) == 2
    assert oracle.iamin(5, x, 1) == 1
    assert oracle.iamax(0, x, 1) == 2**31 - 1
    assert oracle.iamin(3, np.array([np.inf, np.inf, np.inf]), 1) == 2**31 - 1
    assert oracle.iamax(4, x, -1) == 0


@pytest.fixture(scope="module")
def cblas():
    try:
        return oracle.CBlas()
    except OSError as e:
        pytest.skip(str(e))


@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
def test_oracle_gemm_vs_cblas(cblas, ta, tb):
    g = rng(1)
    m, n, k = 63, 45, 37
    lda, ldb, ldc = (k if ta else m) + 3, (n if tb else k) + 1, m + 2
    a = g.uniform(-1, 1, lda * (m if ta else k)).astype(np.float32)
    b = g.uniform(-1, 1, ldb * (k if tb else n)).astype(np.float32)
    c = g.uniform(-1, 1, ldc * n).astype(np.float32)
    ref = c.copy()
    cblas.sgemm(ta, tb, m, n, k, 1.5, a, lda, b, ldb, 0.5, ref, ldc)
    full = oracle.gemm(ta, tb, m, n, k, 1.5, a, lda, b, ldb, 0.5, c, ldc)
    got = ref.reshape(n, ldc).T[:m]
    np.testing.assert_allclose(got, full, rtol=1e-4, atol=1e-4)
    fo = oracle.sgemm_reforder(ta, tb, m, n, k, 1.5, a, lda, b, ldb, 0.5, c, ldc, mode=1)
    assert_almost_equal(fo.reshape(n, ldc).T[:m], full)


def test_oracle_gemm_sampled_entries_match_full():
    g = rng(2)
    m, n, k = 40, 30, 20
    a, b, c = g.standard_normal(m * k), g.standard_normal(k * n), g.standard_normal(m * n)
    full = oracle.gemm(False, False, m, n, k, 1.0, a, m, b, k, 1.0, c, m)
    rows, cols = g.integers(0, m, 50), g.integers(0, n, 50)
    part = oracle.gemm(False, False, m, n, k, 1.0, a, m, b, k, 1.0, c, m, rows=rows, cols=cols)
    np.testing.assert_array_equal(part, full[rows, cols])


@pytest.mark.parametrize("inc", [1, 3])
def test_oracle_blas1_vs_cblas(cblas, inc):
    g = rng(3)
    n = 10007
    x = g.standard_normal(n * inc).astype(np.float32)
    y = g.standard_normal(n * inc).astype(np.float32)
    assert oracle.asum(n, x, inc) == pytest.approx(cblas.sasum(n, x, inc), rel=1e-5)
    assert oracle.nrm2(n, x, inc) == pytest.approx(cblas.snrm2(n, x, inc), rel=1e-5)
    assert oracle.dot(n, x, inc, y, inc) == pytest.approx(cblas.sdot(n, x, inc, y, inc), rel=1e-3, abs=1e-2)
    assert oracle.iamax(n, x, inc) == cblas.isamax(n, x, inc)
    assert oracle.iamin(n, x, inc) == cblas.isamin(n, x, inc)


@pytest.mark.parametrize("trans", ["n", "t"])
def test_oracle_gemv_vs_cblas(cblas, trans):
    g = rng(4)
    m, n, lda, incx, incy = 1023, 514, 2046, 2, 3
    a = g.uniform(-1, 1, lda * n).astype(np.float32)
    xlen, ylen = (n, m) if trans == "n" else (m, n)
    x = g.uniform(-1, 1, xlen * incx).astype(np.float32)
    y = g.uniform(-1, 1, ylen * incy).astype(np.float32)
    ref = y.copy()
    cblas.sgemv(trans, m, n, 1.5, a, lda, x, incx, 1.5, ref, incy)
    got = oracle.gemv(trans, m, n, 1.5, a, lda, x, incx, 1.5, y, incy)
    np.testing.assert_allclose(ref[::incy][:ylen], got, rtol=1e-4, atol=1e-4)


def test_oracle_gemv_negative_increments():
    g = rng(5)
    m, n = 7, 5
    a = g.standard_normal(m * n)
    x = g.standard_normal(n)
    y = g.standard_normal(m)
    got = oracle.gemv("n", m, n, 1.0, a, m, x, -1, 0.0, y, -1)
    ref = a.reshape(n, m).T @ x[::-1]
    np.testing.assert_allclose(got, ref, rtol=1e-12)


@pytest.mark.parametrize("op", list(oracle.OPS))
@pytest.mark.parametrize("dim", ["inner", "outer"])
def test_oracle_reduction_vs_numpy(op, dim):
    g = rng(6)
    rows, cols, ld = 7, 15, 14
    lo, hi = (-2.0, 1.0) if op == "product" else (-2.0, 5.0)
    full = g.uniform(lo, hi, ld * cols)
    mat = full.reshape(cols, ld).T[:rows]
    axis = 0 if dim == "inner" else 1
    ref = {"add": mat.sum(axis), "product": mat.prod(axis), "max": mat.max(axis), "min": mat.min(axis),
           "abs_add": np.abs(mat).sum(axis), "mean": mat.mean(axis)}[op]
    got = oracle.reduction(op, dim, full, ld, rows, cols)
    np.testing.assert_allclose(got, ref, rtol=1e-12)


@pytest.mark.parametrize("incx,incy", [(1, 1), (2, 3), (3, -2)])
def test_oracle_axpy_copy_vs_cblas(cblas, incx, incy):
    """_axpy and _copy restatements against CBLAS on strided views (negative
    increments walk the vector from its end, as in portBLAS's VectorView)."""
    g = rng(5)
    n = 1001
    x = g.standard_normal(n * abs(incx)).astype(np.float32)
    y = g.standard_normal(n * abs(incy)).astype(np.float32)
    ref = y.copy()
    cblas.saxpy(n, 0.75, x, incx, ref, incy)
    np.testing.assert_allclose(oracle.axpy(n, 0.75, x, incx, y, incy), ref, rtol=1e-6, atol=1e-6)
    ref = y.copy()
    cblas.scopy(n, x, incx, ref, incy)
    np.testing.assert_array_equal(oracle.copy(n, x, incx, y, incy).astype(np.float32), ref)


@pytest.mark.parametrize("inc", [1, 4])
def test_oracle_scal_sdsdot_vs_cblas(cblas, inc):
    g = rng(6)
    n = 777
    x = g.standard_normal(n * inc).astype(np.float32)
    y = g.standard_normal(n * inc).astype(np.float32)
    ref = x.copy()
    cblas.sscal(n, -1.25, ref, inc)
    np.testing.assert_allclose(oracle.scal(n, -1.25, x, inc), ref, rtol=1e-6, atol=0)
    # alpha == 0 writes zeros, the value of x notwithstanding
    ref = x.copy()
    cblas.sscal(n, 0.0, ref, inc)
    np.testing.assert_array_equal(oracle.scal(n, 0.0, x, inc).astype(np.float32), ref)
    got = oracle.sdsdot(n, 0.5, x, inc, y, inc)
    assert got == pytest.approx(cblas.sdsdot(n, 0.5, x, inc, y, inc), rel=1e-5, abs=1e-4)
    assert oracle.sdsdot(0, 0.5, x, inc, y, inc) == 0.5


@pytest.mark.parametrize("side,uplo", [("l", "u"), ("l", "l"), ("r", "u"), ("r", "l")])
def test_oracle_symm_vs_cblas(cblas, side, uplo):
    """SYMM reads only the referenced triangle of A; the other triangle holds
    garbage that must not leak into the result."""
    g = rng(7)
    m, n = 37, 23
    na = m if side == "l" else n
    lda, ldb, ldc = na + 2, m + 1, m + 3
    a = g.uniform(-1, 1, lda * na).astype(np.float32)
    b = g.uniform(-1, 1, ldb * n).astype(np.float32)
    c = g.uniform(-1, 1, ldc * n).astype(np.float32)
    ref = c.copy()
    cblas.ssymm(side, uplo, m, n, 1.5, a, lda, b, ldb, 0.5, ref, ldc)
    got = oracle.symm(side, uplo, m, n, 1.5, a, lda, b, ldb, 0.5, c, ldc)
    np.testing.assert_allclose(got, ref.reshape(n, ldc).T[:m], rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("trans", ["n", "t"])
def test_oracle_omatcopy_vs_cblas(cblas, trans):
    g = rng(8)
    m, n = 45, 31
    lda = m + 3
    ldb = (m if trans == "n" else n) + 2
    a = g.uniform(-1, 1, lda * n).astype(np.float32)
    out = g.uniform(-1, 1, ldb * (n if trans == "n" else m)).astype(np.float32)
    ref = out.copy()
    cblas.somatcopy(trans, m, n, 2.0, a, lda, ref, ldb)
    got = oracle.omatcopy(trans, m, n, 2.0, a, lda, out, ldb)
    np.testing.assert_array_equal(got.astype(np.float32), ref)


@pytest.mark.parametrize("dim", ["inner", "outer"])
@pytest.mark.parametrize("rows,cols,ld", [(1, 1, 1), (17, 5, 20), (1000, 37, 1003), (513, 1030, 513)])
def test_cpu_baseline_reduction_matches_fp64(dim, rows, cols, ld):
    """The timed CPU restatement of the Reduction kernel (FP32 lanes + tree)
    agrees with an FP64 sum within FP32 accumulation error."""
    g = np.random.default_rng(rows * 7 + cols)
    a = g.uniform(-1, 1, ld * cols).astype(np.float32)
    got = oracle.cpu_reduction_add(dim, a, ld, rows, cols)
    M = a.reshape(cols, ld)[:, :rows].astype(np.float64)  # M[c, r]
    ref = M.sum(1) if dim == "inner" else M.sum(0)
    n_red = rows if dim == "inner" else cols
    np.testing.assert_allclose(got, ref, rtol=0, atol=4 * n_red * 2.0 ** -24 * np.abs(M).max() + 1e-7)


@pytest.mark.parametrize("n", [1, 2, 1000, 100003])
def test_cpu_baseline_iamax_iamin_first_index(n):
    g = np.random.default_rng(n)
    x = g.standard_normal(n).astype(np.float32)
    if n > 10:
        x[[3, n // 2, n - 1]] = 7.5   # ties: the first index wins
        x[[5, n // 3]] = 0.0
    assert oracle.cpu_iamax(x) == int(np.argmax(np.abs(x)))
    assert oracle.cpu_iamax(x, is_min=True) == int(np.argmin(np.abs(x)))
