"""GPU parity of _gemm / _gemm_batched / _gemm_strided_batched against the
oracle through the C ABI, on portBLAS's sweep
(test/unittest/blas3/blas3_gemm_test.cpp:29-141, blas3_gemm_batched_test.cpp,
verify_gemm in blas3_gemm_common.hpp:96-230), for each FP32 method."""
import json
import os

import numpy as np
import pytest

import oracle
from tests.util import rng, to_dev, to_host, assert_almost_equal

pytestmark = pytest.mark.gpu
KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kat.json")))
MODES = ["fp32_simt", "split_bf16x3", "split_bf16x6"]
U32 = 2.0 ** -24


def norm_bound(mode, k):
    """Componentwise bound on |C - C64| / (|alpha||A||B| + |beta C|): FP32
    accumulation (K u) plus, for the 2-term split, the dropped 2^-16 terms."""
    base = 2.0 * (k + 2) * U32
    return base + (4.0 * 2.0 ** -16 if mode == "split_bf16x3" else 4.0 * U32)


@pytest.fixture(autouse=True)
def _reset_mode(sb):
    yield
    from portblas_gb300 import blas
    sb.set_sgemm_mode(blas.sgemm_mode_t.auto)
    sb.check_device_error()


def _mats(g, ta, tb, m, n, k, lda_mul, ldb_mul, ldc_mul, off, dtype):
    lda = (k if ta else m) * lda_mul
    ldb = (n if tb else k) * ldb_mul
    ldc = m * ldc_mul
    a = g.uniform(-2, 5, off + lda * (m if ta else k)).astype(dtype)
    b = g.uniform(-2, 5, off + ldb * (k if tb else n)).astype(dtype)
    c = g.uniform(-2, 5, off + ldc * n).astype(dtype)
    return a, lda, b, ldb, c, ldc


def _gemm(sb, torch, mode, ta, tb, m, n, k, alpha, beta, lda_mul=1, ldb_mul=1, ldc_mul=1, off=0,
          dtype=np.float32, seed=0, c_nan=False, want_scale=False):
    from portblas_gb300 import blas
    g = rng(seed + m * 3 + n * 5 + k * 7)
    a, lda, b, ldb, c, ldc = _mats(g, ta, tb, m, n, k, lda_mul, ldb_mul, ldc_mul, off, dtype)
    if c_nan:
        c[:] = np.nan
    ref = oracle.gemm(ta, tb, m, n, k, alpha, a[off:], lda, b[off:], ldb, beta, c[off:], ldc)
    if mode is not None:
        sb.set_sgemm_mode(getattr(blas.sgemm_mode_t, mode))
    ad, bd, cd = to_dev(a, torch), to_dev(b, torch), to_dev(c, torch)
    blas._gemm(sb, "t" if ta else "n", "t" if tb else "n", m, n, k, alpha, ad[off:], lda, bd[off:], ldb, beta,
               cd[off:], ldc)
    out = to_host(cd)
    got = out[off:off + ldc * n].reshape(n, ldc).T[:m]
    # bytes outside the m x n window must be untouched
    full = c.copy()
    win = full[off:off + ldc * n].reshape(n, ldc).T
    win[:m] = got
    np.testing.assert_array_equal(np.isnan(out), np.isnan(full))
    np.testing.assert_array_equal(np.nan_to_num(out), np.nan_to_num(full))
    if want_scale:
        scale = oracle.gemm_absscale(ta, tb, m, n, k, alpha, a[off:], lda, b[off:], ldb, beta, c[off:], ldc)
        return got, ref, scale
    return got, ref


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
@pytest.mark.parametrize("m,n,k", [(11, 11, 16), (16, 63, 17), (63, 16, 63), (253, 32, 253), (32, 253, 511),
                                   (129, 257, 64)])
@pytest.mark.parametrize("alpha,beta", [(1.5, 0.0), (1.0, 1.0), (1.5, 1.5), (0.0, 1.5)])
def test_gemm_sweep(sb, torch_cuda, mode, ta, tb, m, n, k, alpha, beta):
    got, ref, scale = _gemm(sb, torch_cuda, mode, ta, tb, m, n, k, alpha, beta, want_scale=True)
    assert_almost_equal(got, ref)
    err = np.abs(got - ref) / np.maximum(scale, 1e-300)
    assert err.max() <= norm_bound(mode, k), (mode, float(err.max()))


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("lda_mul,ldb_mul,ldc_mul,off", [(2, 3, 4, 0), (1, 1, 1, 1), (3, 2, 1, 10)])
@pytest.mark.parametrize("ta,tb", [(False, False), (True, True)])
def test_gemm_ld_and_offsets(sb, torch_cuda, mode, lda_mul, ldb_mul, ldc_mul, off, ta, tb):
    got, ref = _gemm(sb, torch_cuda, mode, ta, tb, 63, 45, 37, 1.5, 0.5, lda_mul, ldb_mul, ldc_mul, off)
    assert_almost_equal(got, ref)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("alpha", [1.0, 0.0])
def test_gemm_beta0_never_reads_c(sb, torch_cuda, mode, alpha):
    got, ref = _gemm(sb, torch_cuda, mode, False, False, 33, 17, 9, alpha, 0.0, c_nan=True)
    assert np.all(np.isfinite(got))
    assert_almost_equal(got, ref)


@pytest.mark.parametrize("case", KAT["gemm"], ids=lambda c: f"{c['ta']}{c['tb']}-a{c['alpha']}-b{c['beta']}")
def test_gemm_kat(sb, torch_cuda, case):
    torch = torch_cuda
    from portblas_gb300 import blas
    c = np.array(case["c"], dtype=np.float32)
    if case["c_nan"]:
        c[:] = np.nan
    cd = to_dev(c, torch)
    blas._gemm(sb, case["ta"], case["tb"], case["m"], case["n"], case["k"], case["alpha"],
               to_dev(np.array(case["a"], dtype=np.float32), torch), case["lda"],
               to_dev(np.array(case["b"], dtype=np.float32), torch), case["ldb"], case["beta"], cd, case["ldc"])
    np.testing.assert_array_equal(to_host(cd), np.array(case["expected"], dtype=np.float32))


def test_gemm_invalid_trans_raises(sb, torch_cuda):
    torch = torch_cuda
    from portblas_gb300 import blas
    x = torch.zeros(16, device="cuda")
    with pytest.raises(blas.InvalidArgument, match="_TransA"):
        blas._gemm(sb, "x", "n", 4, 4, 4, 1.0, x, 4, x, 4, 0.0, x, 4)
    with pytest.raises(blas.InvalidArgument, match="_TransB"):
        blas._gemm(sb, "n", "q", 4, 4, 4, 1.0, x, 4, x, 4, 0.0, x, 4)
    # alpha == 0 skips trans validation (gemm_interface.hpp:112-139)
    blas._gemm(sb, "x", "n", 4, 4, 4, 0.0, x, 4, x, 4, 0.0, x, 4)


def test_gemm_strided_invalid_strides(sb, torch_cuda):
    torch = torch_cuda
    from portblas_gb300 import blas
    x = torch.zeros(1024, device="cuda")
    with pytest.raises(blas.InvalidArgument, match="_stridec"):
        blas._gemm_strided_batched(sb, "n", "n", 4, 4, 4, 1.0, x, 4, 16, x, 4, 16, 0.0, x, 4, 15, 2)
    with pytest.raises(blas.InvalidArgument, match="_stridea"):
        blas._gemm_strided_batched(sb, "n", "n", 4, 4, 4, 1.0, x, 4, -1, x, 4, 16, 0.0, x, 4, 16, 2)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True)])
@pytest.mark.parametrize("beta", [0.0, 1.5])
def test_gemm_batched_default_strides(sb, torch_cuda, mode, ta, tb, beta):
    torch = torch_cuda
    from portblas_gb300 import blas
    sb.set_sgemm_mode(getattr(blas.sgemm_mode_t, mode))
    g = rng(17)
    m, n, k, batch = 37, 29, 23, 5
    lda, ldb, ldc = (k if ta else m), (n if tb else k), m
    sa, sbb, sc = (m * lda if ta else k * lda), (ldb * k if tb else n * ldb), ldc * n
    a = g.uniform(-2, 5, sa * batch).astype(np.float32)
    b = g.uniform(-2, 5, sbb * batch).astype(np.float32)
    c = g.uniform(-2, 5, sc * batch).astype(np.float32)
    cd = to_dev(c, torch)
    blas._gemm_batched(sb, "t" if ta else "n", "t" if tb else "n", m, n, k, 1.5, to_dev(a, torch), lda,
                       to_dev(b, torch), ldb, beta, cd, ldc, batch)
    out = to_host(cd)
    for i in range(batch):
        ref = oracle.gemm(ta, tb, m, n, k, 1.5, a[i * sa:], lda, b[i * sbb:], ldb, beta, c[i * sc:], ldc)
        assert_almost_equal(out[i * sc:(i + 1) * sc].reshape(n, ldc).T[:m], ref)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("stride_mul", [1, 2])
def test_gemm_strided_batched(sb, torch_cuda, mode, stride_mul):
    torch = torch_cuda
    from portblas_gb300 import blas
    sb.set_sgemm_mode(getattr(blas.sgemm_mode_t, mode))
    g = rng(19)
    m, n, k, batch = 64, 64, 64, 7
    sa, sbb, sc = m * k * stride_mul, 0, m * n * stride_mul  # stride_b == 0 shares B
    a = g.uniform(-1, 1, sa * batch).astype(np.float32)
    b = g.uniform(-1, 1, k * n).astype(np.float32)
    c = g.uniform(-1, 1, sc * batch).astype(np.float32)
    cd = to_dev(c, torch)
    blas._gemm_strided_batched(sb, "n", "n", m, n, k, 1.0, to_dev(a, torch), m, sa, to_dev(b, torch), k, sbb, 0.5,
                               cd, m, sc, batch)
    out = to_host(cd)
    for i in range(batch):
        ref = oracle.gemm(False, False, m, n, k, 1.0, a[i * sa:], m, b, k, 0.5, c[i * sc:], m)
        assert_almost_equal(out[i * sc:i * sc + m * n].reshape(n, m).T, ref)
        if stride_mul > 1:  # gap between matrices untouched
            np.testing.assert_array_equal(out[i * sc + m * n:(i + 1) * sc], c[i * sc + m * n:(i + 1) * sc])


@pytest.mark.parametrize("ta,tb", [(False, False), (True, False)])
def test_dgemm(sb, torch_cuda, ta, tb):
    got, ref = _gemm(sb, torch_cuda, None, ta, tb, 129, 65, 257, 1.5, 0.5, dtype=np.float64)
    assert_almost_equal(got, ref, dtype=np.float64)


def test_dgemm_strided_batched(sb, torch_cuda):
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(23)
    m = n = k = 33
    batch = 3
    a = g.uniform(-1, 1, m * k * batch)
    b = g.uniform(-1, 1, k * n * batch)
    c = np.zeros(m * n * batch)
    cd = to_dev(c, torch)
    blas._gemm_strided_batched(sb, "n", "t", m, n, k, 1.0, to_dev(a, torch), m, m * k, to_dev(b, torch), n, k * n,
                               0.0, cd, m, m * n, batch)
    out = to_host(cd)
    for i in range(batch):
        ref = oracle.gemm(False, True, m, n, k, 1.0, a[i * m * k:], m, b[i * k * n:], n, 0.0, None, m)
        assert_almost_equal(out[i * m * n:(i + 1) * m * n].reshape(n, m).T, ref, dtype=np.float64)


@pytest.mark.parametrize("ta", [False, True])
def test_split_bf16x6_is_fp32_accurate(sb, torch_cuda, ta):
    """The 3-term split with chunked tensor-memory accumulation, its leading
    products kept in their own accumulator, is at least as accurate as plain
    FP32 on wide-range data (entries s*2^u, u ~ U[-10, 10]) at K = 4096,
    measured against the FP64 oracle."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(41)
    m = n = 256
    k = 4096
    a = (g.choice([-1.0, 1.0], m * k) * np.exp2(g.uniform(-10, 10, m * k))).astype(np.float32)
    b = (g.choice([-1.0, 1.0], k * n) * np.exp2(g.uniform(-10, 10, k * n))).astype(np.float32)
    lda = k if ta else m
    ref = oracle.gemm(ta, False, m, n, k, 1.0, a, lda, b, k, 0.0, None, m)
    scale = oracle.gemm_absscale(ta, False, m, n, k, 1.0, a, lda, b, k, 0.0, None, m)
    errs = {}
    for mode in ("fp32_simt", "split_bf16x6", "split_bf16x3"):
        sb.set_sgemm_mode(getattr(blas.sgemm_mode_t, mode))
        cd = torch.zeros(m * n, device="cuda")
        blas._gemm(sb, "t" if ta else "n", "n", m, n, k, 1.0, to_dev(a, torch), lda, to_dev(b, torch), k, 0.0, cd, m)
        got = to_host(cd).reshape(n, m).T
        e = np.abs(got - ref) / scale
        errs[mode] = (float(e.mean()), float(e.max()))
    simt_mean, simt_max = errs["fp32_simt"]
    x6_mean, x6_max = errs["split_bf16x6"]
    assert x6_mean <= simt_mean, errs
    assert x6_max <= simt_max, errs
    assert errs["split_bf16x3"][1] <= 6e-5, errs  # the dropped 2^-16 terms bound the 2-term split


def _to_interleaved(mats, ld_rows, ld_cols):
    """Batch-fastest layout of a list of column-major ld_rows x ld_cols
    matrices: element (r, c) of matrix b at [(r + c*ld_rows)*batch + b]
    (test/unittest/blas3/blas3_gemm_common.hpp:53-69)."""
    stack = np.stack([m[: ld_rows * ld_cols] for m in mats])  # [batch][ld_rows*ld_cols]
    return np.ascontiguousarray(stack.T).ravel()


@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
@pytest.mark.parametrize("m,n,k,batch", [(4, 4, 4, 1000), (5, 3, 7, 129), (16, 20, 9, 64)])
@pytest.mark.parametrize("alpha,beta", [(1.5, 0.5), (1.0, 0.0), (0.0, 2.0)])
def test_gemm_batched_interleaved(sb, torch_cuda, ta, tb, m, n, k, batch, alpha, beta):
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(m + n + k + batch)
    lda, ldb, ldc = (k if ta else m), (n if tb else k), m
    acols, bcols = (m if ta else k), (k if tb else n)
    As = [g.uniform(-2, 5, lda * acols).astype(np.float32) for _ in range(batch)]
    Bs = [g.uniform(-2, 5, ldb * bcols).astype(np.float32) for _ in range(batch)]
    Cs = [g.uniform(-2, 5, ldc * n).astype(np.float32) for _ in range(batch)]
    cd = to_dev(_to_interleaved(Cs, ldc, n), torch)
    blas._gemm_batched(sb, "t" if ta else "n", "t" if tb else "n", m, n, k, alpha,
                       to_dev(_to_interleaved(As, lda, acols), torch), lda,
                       to_dev(_to_interleaved(Bs, ldb, bcols), torch), ldb, beta, cd, ldc, batch,
                       blas.gemm_batch_type_t.interleaved)
    out = to_host(cd).reshape(ldc * n, batch).T  # back to [batch][ldc*n]
    for i in range(0, batch, max(1, batch // 7)):
        ref = oracle.gemm(ta, tb, m, n, k, alpha, As[i], lda, Bs[i], ldb, beta, Cs[i], ldc)
        assert_almost_equal(out[i].reshape(n, ldc).T[:m], ref)


@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
@pytest.mark.parametrize("m,n,k", [(64, 64, 64), (7, 33, 64), (64, 1, 17), (50, 60, 3)])
@pytest.mark.parametrize("beta", [0.0, 0.75])
def test_gemm_strided_small_batch_path(sb, torch_cuda, ta, tb, m, n, k, beta):
    """Many small problems take the one-CTA-per-problem kernel under AUTO."""
    torch = torch_cuda
    from portblas_gb300 import blas
    sb.set_sgemm_mode(blas.sgemm_mode_t.auto)
    g = rng(m * n + k)
    batch = 700
    lda, ldb, ldc = (k if ta else m) + 1, (n if tb else k) + 2, m + 3
    sa, sbs, sc = lda * (m if ta else k) + 5, ldb * (k if tb else n), ldc * n + 1
    a = g.uniform(-1, 1, sa * batch).astype(np.float32)
    b = g.uniform(-1, 1, sbs * batch).astype(np.float32)
    c = g.uniform(-1, 1, sc * batch).astype(np.float32)
    cd = to_dev(c, torch)
    blas._gemm_strided_batched(sb, "t" if ta else "n", "t" if tb else "n", m, n, k, 1.25, to_dev(a, torch), lda, sa,
                               to_dev(b, torch), ldb, sbs, beta, cd, ldc, sc, batch)
    out = to_host(cd)
    for i in (0, 1, 350, batch - 1):
        ref = oracle.gemm(ta, tb, m, n, k, 1.25, a[i * sa:], lda, b[i * sbs:], ldb, beta, c[i * sc:], ldc)
        got = out[i * sc:i * sc + ldc * n].reshape(n, ldc).T[:m]
        assert_almost_equal(got, ref)
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5 * k)
        np.testing.assert_array_equal(out[i * sc:i * sc + ldc * n].reshape(n, ldc).T[m:],
                                      c[i * sc:i * sc + ldc * n].reshape(n, ldc).T[m:])


@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
@pytest.mark.parametrize("m,n,k", [(64, 64, 64), (32, 48, 16), (8, 4, 12)])
def test_gemm_strided_small_batch_vector_loads(sb, torch_cuda, ta, tb, m, n, k):
    """Small-batch kernel with 16-byte-aligned operands (the 128-bit load
    path): exact leading dimensions and strides that are multiples of 4."""
    torch = torch_cuda
    from portblas_gb300 import blas
    sb.set_sgemm_mode(blas.sgemm_mode_t.auto)
    g = rng(7 * m + n + k)
    batch = 640
    lda, ldb, ldc = (k if ta else m), (n if tb else k), m
    sa, sbs, sc = lda * (m if ta else k), ldb * (k if tb else n), ldc * n
    a = g.uniform(-1, 1, sa * batch).astype(np.float32)
    b = g.uniform(-1, 1, sbs * batch).astype(np.float32)
    c = g.uniform(-1, 1, sc * batch).astype(np.float32)
    cd = to_dev(c, torch)
    blas._gemm_strided_batched(sb, "t" if ta else "n", "t" if tb else "n", m, n, k, 1.0, to_dev(a, torch), lda, sa,
                               to_dev(b, torch), ldb, sbs, 0.5, cd, ldc, sc, batch)
    out = to_host(cd)
    for i in (0, 3, 333, batch - 1):
        ref = oracle.gemm(ta, tb, m, n, k, 1.0, a[i * sa:], lda, b[i * sbs:], ldb, 0.5, c[i * sc:], ldc)
        got = out[i * sc:(i + 1) * sc].reshape(n, ldc).T
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5 * k)


@pytest.mark.parametrize("mode", ["auto", "fp32_simt", "split_bf16x6"])
def test_gemm_tall_skinny_split_k(sb, torch_cuda, mode):
    """Tall-skinny reduction-dimension shapes (M = N = 48, K = 2^18) take the
    split-K partial + reduction path; sampled entries against the FP64 oracle
    within the FP32 accumulation bound."""
    torch = torch_cuda
    from portblas_gb300 import blas
    sb.set_sgemm_mode(getattr(blas.sgemm_mode_t, mode))
    g = rng(99)
    m = n = 48
    k = 1 << 18
    a = g.uniform(-1, 1, m * k).astype(np.float32)
    b = g.uniform(-1, 1, k * n).astype(np.float32)
    cd = torch.zeros(m * n, device="cuda")
    blas._gemm(sb, "n", "n", m, n, k, 1.0, to_dev(a, torch), m, to_dev(b, torch), k, 0.0, cd, m)
    got = to_host(cd).reshape(n, m).T
    rows = g.integers(0, m, 24)
    cols = g.integers(0, n, 24)
    ref = oracle.gemm(False, False, m, n, k, 1.0, a, m, b, k, 0.0, None, m, rows=rows, cols=cols)
    scale = oracle.gemm_absscale(False, False, m, n, k, 1.0, a, m, b, k, 0.0, None, m, rows=rows, cols=cols)
    err = np.abs(got[rows, cols] - ref) / scale
    assert err.max() <= 2.0 * (k + 4) * 2.0 ** -24, err.max()
    sb.set_sgemm_mode(blas.sgemm_mode_t.auto)


@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
@pytest.mark.parametrize("m,n,k,beta", [(64, 64, 64, 0.0), (40, 24, 52, 0.5)])
def test_gemm_strided_small_batch_tensor_cores(sb, torch_cuda, ta, tb, m, n, k, beta):
    """The tensor-core small-batch path (16-byte-aligned layouts, two
    problems per tile): an odd batch, so the last tile holds one problem and
    a zero-filled one; every problem's C against FP64 at FP32-level accuracy
    (|A||B|-normalised), the neighbouring padding of C untouched."""
    torch = torch_cuda
    from portblas_gb300 import blas
    sb.set_sgemm_mode(blas.sgemm_mode_t.auto)
    g = rng(11 * m + 3 * n + k)
    batch = 611
    lda, ldb, ldc = (k if ta else m) + 4, (n if tb else k) + 8, m + 1
    sa, sbs, sc = lda * (m if ta else k), ldb * (k if tb else n) + 4, ldc * n + 3
    a = g.uniform(-1, 1, sa * batch).astype(np.float32)
    b = g.uniform(-1, 1, sbs * batch).astype(np.float32)
    c = g.uniform(-1, 1, sc * batch).astype(np.float32)
    cd = to_dev(c, torch)
    blas._gemm_strided_batched(sb, "t" if ta else "n", "t" if tb else "n", m, n, k, 1.5, to_dev(a, torch), lda, sa,
                               to_dev(b, torch), ldb, sbs, beta, cd, ldc, sc, batch)
    out = to_host(cd)
    for i in (0, 1, 2, 305, batch - 2, batch - 1):
        ref = oracle.gemm(ta, tb, m, n, k, 1.5, a[i * sa:], lda, b[i * sbs:], ldb, beta, c[i * sc:], ldc)
        scale = oracle.gemm_absscale(ta, tb, m, n, k, 1.5, a[i * sa:], lda, b[i * sbs:], ldb, beta, c[i * sc:], ldc)
        blk = out[i * sc:i * sc + ldc * n].reshape(n, ldc).T
        got = blk[:m]
        assert (np.abs(got - ref) / scale).max() <= 2.0 * (k + 2) * U32, i
        np.testing.assert_array_equal(blk[m:], c[i * sc:i * sc + ldc * n].reshape(n, ldc).T[m:])
        np.testing.assert_array_equal(out[i * sc + ldc * n:(i + 1) * sc], c[i * sc + ldc * n:(i + 1) * sc])
    sb.check_device_error()


@pytest.mark.parametrize("mode", ["split_bf16x3", "split_bf16x6"])
@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
def test_split_bf16_cta_pair_256_tiles(sb, torch_cuda, ta, tb, mode):
    """x3 and x6 on 256 x 256 CTA-pair tiles (taken when M and N are at
    least 256 and the tiles fill half of the resident clusters): M and N not
    multiples of 256, K of two or
    three TMEM chunks and a ragged last k-block, a strided batch, alpha and
    beta; against the oracle at the mode's bound, and the rows and columns
    outside each C untouched."""
    torch = torch_cuda
    from portblas_gb300 import blas
    sb.set_sgemm_mode(getattr(blas.sgemm_mode_t, mode))
    m, n, k, batch = 1000, 1000, 300, 40  # 4 x 4 x 40 = 640 tiles of 256 x 256
    g = rng(m + n + k + int(ta) * 2 + int(tb) + 7)
    lda, ldb, ldc = (k if ta else m) + 3, (n if tb else k) + 5, m + 7
    sa, sbs, sc = lda * (m if ta else k), ldb * (k if tb else n), ldc * n + 11
    a = g.uniform(-1, 1, sa * batch).astype(np.float32)
    b = g.uniform(-1, 1, sbs * batch).astype(np.float32)
    c = g.uniform(-1, 1, sc * batch).astype(np.float32)
    cd = to_dev(c, torch)
    blas._gemm_strided_batched(sb, "t" if ta else "n", "t" if tb else "n", m, n, k, 0.75, to_dev(a, torch), lda, sa,
                               to_dev(b, torch), ldb, sbs, 1.5, cd, ldc, sc, batch)
    out = to_host(cd)
    for i in (0, 17, batch - 1):
        ref = oracle.gemm(ta, tb, m, n, k, 0.75, a[i * sa:], lda, b[i * sbs:], ldb, 1.5, c[i * sc:], ldc)
        scale = oracle.gemm_absscale(ta, tb, m, n, k, 0.75, a[i * sa:], lda, b[i * sbs:], ldb, 1.5, c[i * sc:],
                                     ldc)
        blk = out[i * sc:i * sc + ldc * n].reshape(n, ldc).T
        assert (np.abs(blk[:m] - ref) / scale).max() <= norm_bound(mode, k), i
        np.testing.assert_array_equal(blk[m:], c[i * sc:i * sc + ldc * n].reshape(n, ldc).T[m:])
        np.testing.assert_array_equal(out[i * sc + ldc * n:(i + 1) * sc], c[i * sc + ldc * n:(i + 1) * sc])
    sb.check_device_error()


@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
def test_split_bf16x3_cta_pair_tiles(sb, torch_cuda, ta, tb):
    """x3 on 256 x 128 CTA-pair tiles (taken when N is below 256, which
    rules out 256 x 256 tiles, and there are at least two waves of 128 x 128
    tiles): M not a multiple of 256, ragged N and K, a strided batch, alpha
    and beta; against the oracle at the x3 bound, and the rows and columns
    outside each C untouched."""
    torch = torch_cuda
    from portblas_gb300 import blas
    sb.set_sgemm_mode(blas.sgemm_mode_t.split_bf16x3)
    m, n, k, batch = 1000, 200, 300, 20  # 8 x 2 x 20 = 320 tiles of 128 x 128
    g = rng(m + n + k + int(ta) * 2 + int(tb))
    lda, ldb, ldc = (k if ta else m) + 3, (n if tb else k) + 5, m + 7
    sa, sbs, sc = lda * (m if ta else k), ldb * (k if tb else n), ldc * n + 11
    a = g.uniform(-1, 1, sa * batch).astype(np.float32)
    b = g.uniform(-1, 1, sbs * batch).astype(np.float32)
    c = g.uniform(-1, 1, sc * batch).astype(np.float32)
    cd = to_dev(c, torch)
    blas._gemm_strided_batched(sb, "t" if ta else "n", "t" if tb else "n", m, n, k, 1.25, to_dev(a, torch), lda, sa,
                               to_dev(b, torch), ldb, sbs, -0.5, cd, ldc, sc, batch)
    out = to_host(cd)
    for i in (0, 3, batch - 1):
        ref = oracle.gemm(ta, tb, m, n, k, 1.25, a[i * sa:], lda, b[i * sbs:], ldb, -0.5, c[i * sc:], ldc)
        scale = oracle.gemm_absscale(ta, tb, m, n, k, 1.25, a[i * sa:], lda, b[i * sbs:], ldb, -0.5, c[i * sc:],
                                     ldc)
        blk = out[i * sc:i * sc + ldc * n].reshape(n, ldc).T
        assert (np.abs(blk[:m] - ref) / scale).max() <= norm_bound("split_bf16x3", k), i
        np.testing.assert_array_equal(blk[m:], c[i * sc:i * sc + ldc * n].reshape(n, ldc).T[m:])
        np.testing.assert_array_equal(out[i * sc + ldc * n:(i + 1) * sc], c[i * sc + ldc * n:(i + 1) * sc])
    sb.check_device_error()


@pytest.mark.parametrize("m,n,k,batch", [(512, 512, 512, 16), (2000, 1500, 300, 1)])
def test_auto_on_pair_tile_shapes(sb, torch_cuda, m, n, k, batch):
    """AUTO sends shapes that fit 256 x 256 CTA-pair tiles (M, N >= 256,
    enough tiles, rounds well filled) to the x6 split: a strided batch and a
    single problem whose tiles stay partly outside it, alpha and beta, every
    entry of sampled matrices against the oracle at the x6 bound."""
    torch = torch_cuda
    from portblas_gb300 import blas
    sb.set_sgemm_mode(blas.sgemm_mode_t.auto)
    g = rng(m + n + k + batch)
    lda, ldb, ldc = m + 1, k + 2, m + 3
    sa, sbs, sc = lda * k, ldb * n, ldc * n
    a = g.uniform(-1, 1, sa * batch).astype(np.float32)
    b = g.uniform(-1, 1, sbs * batch).astype(np.float32)
    c = g.uniform(-1, 1, sc * batch).astype(np.float32)
    cd = to_dev(c, torch)
    blas._gemm_strided_batched(sb, "n", "n", m, n, k, 1.25, to_dev(a, torch), lda, sa, to_dev(b, torch), ldb, sbs,
                               -0.5, cd, ldc, sc, batch)
    out = to_host(cd)
    for i in sorted({0, batch // 2, batch - 1}):
        ref = oracle.gemm(False, False, m, n, k, 1.25, a[i * sa:], lda, b[i * sbs:], ldb, -0.5, c[i * sc:], ldc)
        scale = oracle.gemm_absscale(False, False, m, n, k, 1.25, a[i * sa:], lda, b[i * sbs:], ldb, -0.5,
                                     c[i * sc:], ldc)
        blk = out[i * sc:(i + 1) * sc].reshape(n, ldc).T
        assert (np.abs(blk[:m] - ref) / scale).max() <= norm_bound("split_bf16x6", k), i
        np.testing.assert_array_equal(blk[m:], c[i * sc:(i + 1) * sc].reshape(n, ldc).T[m:])
    sb.check_device_error()
