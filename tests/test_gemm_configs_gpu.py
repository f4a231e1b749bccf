"""Every FP32 GEMM configuration the selector can pick (SIMT tiles x split-K,
split-BF16 tcgen05 N tiles x split-K x raster) against the oracle, including
strided batches, ragged tiles and both transposes."""
import numpy as np
import pytest

import oracle
from tests.util import rng, assert_almost_equal

pytestmark = pytest.mark.gpu

SHAPES = [  # m, n, k, batch, ta, tb
    (1, 1, 1, 1, False, False),
    (37, 71, 129, 1, False, True),
    (130, 66, 1000, 3, True, False),
    (256, 300, 64, 1, True, True),
    (5, 700, 4100, 2, False, False),
]


@pytest.mark.parametrize("cfg", range(40))
def test_every_config(sb, torch_cuda, cfg):
    torch = torch_cuda
    from portblas_gb300 import _lib
    L = _lib.load()
    for (m, n, k, batch, ta, tb) in SHAPES:
        g = rng(m + n + k + batch + cfg)
        lda, ldb, ldc = (k if ta else m) + 1, (n if tb else k) + 2, m + 3
        sa, sbs, sc = lda * (m if ta else k), ldb * (k if tb else n), ldc * n
        a = g.uniform(-1, 1, sa * batch).astype(np.float32)
        b = g.uniform(-1, 1, sbs * batch).astype(np.float32)
        c = g.uniform(-1, 1, sc * batch).astype(np.float32)
        cd = torch.from_numpy(c.copy()).cuda()
        ad, bd = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        st = L.gbblas_sgemm_strided_batched_config(sb.handle, cfg, b"t" if ta else b"n", b"t" if tb else b"n", m,
                                                   n, k, 1.5, ad.data_ptr(), lda, sa, bd.data_ptr(), ldb, sbs, 0.5,
                                                   cd.data_ptr(), ldc, sc, batch)
        assert st == 0, (cfg, m, n, k, L.gbblas_last_error())
        out = cd.cpu().numpy()
        for i in range(batch):
            ref = oracle.gemm(ta, tb, m, n, k, 1.5, a[i * sa:], lda, b[i * sbs:], ldb, 0.5, c[i * sc:], ldc)
            scale = oracle.gemm_absscale(ta, tb, m, n, k, 1.5, a[i * sa:], lda, b[i * sbs:], ldb, 0.5, c[i * sc:],
                                         ldc)
            got = out[i * sc:(i + 1) * sc].reshape(n, ldc).T[:m]
            assert_almost_equal(got, ref)
            assert (np.abs(got - ref) / scale).max() <= 2.0 * (k + 4) * 2.0 ** -24, (cfg, m, n, k)
            # padding rows between columns untouched
            np.testing.assert_array_equal(out[i * sc:(i + 1) * sc].reshape(n, ldc).T[m:],
                                          c[i * sc:(i + 1) * sc].reshape(n, ldc).T[m:])
    sb.check_device_error()


def test_autotune_and_auto_use_winner(sb, torch_cuda):
    import ctypes as C
    from portblas_gb300 import _lib
    L = _lib.load()
    best, ms = C.c_int(), C.c_float()
    assert L.gbblas_sgemm_autotune(sb.handle, b"n", b"n", 96, 80, 512, 96, 512, 96, 1, 2, C.byref(best),
                                   C.byref(ms)) == 0
    assert 0 <= best.value < 40 and ms.value > 0
    pick = C.c_int()
    assert L.gbblas_sgemm_selector_pick(96, 80, 512, b"n", b"n", 96, 512, 96, 1, C.byref(pick)) == 0
    assert pick.value == best.value


@pytest.mark.parametrize("cfg", range(40, 60))
def test_every_fp64_config(sb, torch_cuda, cfg):
    """The FP64 configs (SIMT tiles x split-K) against the oracle."""
    torch = torch_cuda
    from portblas_gb300 import _lib
    L = _lib.load()
    for (m, n, k, batch, ta, tb) in SHAPES:
        g = rng(m + n + k + batch + cfg)
        lda, ldb, ldc = (k if ta else m) + 1, (n if tb else k) + 2, m + 3
        sa, sbs, sc = lda * (m if ta else k), ldb * (k if tb else n), ldc * n
        a = g.uniform(-1, 1, sa * batch)
        b = g.uniform(-1, 1, sbs * batch)
        c = g.uniform(-1, 1, sc * batch)
        cd = torch.from_numpy(c.copy()).cuda()
        ad, bd = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        st = L.gbblas_dgemm_strided_batched_config(sb.handle, cfg, b"t" if ta else b"n", b"t" if tb else b"n", m,
                                                   n, k, 1.5, ad.data_ptr(), lda, sa, bd.data_ptr(), ldb, sbs, 0.5,
                                                   cd.data_ptr(), ldc, sc, batch)
        assert st == 0, (cfg, m, n, k, L.gbblas_last_error())
        out = cd.cpu().numpy()
        for i in range(batch):
            ref = oracle.gemm(ta, tb, m, n, k, 1.5, a[i * sa:], lda, b[i * sbs:], ldb, 0.5, c[i * sc:], ldc)
            got = out[i * sc:(i + 1) * sc].reshape(n, ldc).T[:m]
            assert_almost_equal(got, ref, dtype=np.float64)
            np.testing.assert_array_equal(out[i * sc:(i + 1) * sc].reshape(n, ldc).T[m:],
                                          c[i * sc:(i + 1) * sc].reshape(n, ldc).T[m:])
    # FP32 entry points refuse FP64 configs and the other way round
    buf = torch.zeros(16, device="cuda", dtype=torch.float64)
    assert L.gbblas_dgemm_strided_batched_config(sb.handle, 3, b"n", b"n", 2, 2, 2, 1.0, buf.data_ptr(), 2, 4,
                                                 buf.data_ptr(), 2, 4, 0.0, buf.data_ptr(), 2, 4, 1) == 1
    sb.check_device_error()


def test_dgemm_autotune_and_auto_use_winner(sb, torch_cuda):
    import ctypes as C
    from portblas_gb300 import _lib
    L = _lib.load()
    best, ms = C.c_int(), C.c_float()
    assert L.gbblas_dgemm_autotune(sb.handle, b"t", b"n", 96, 80, 512, 512, 512, 96, 1, 2, C.byref(best),
                                   C.byref(ms)) == 0
    assert 40 <= best.value < 60 and ms.value > 0
    pick = C.c_int()
    assert L.gbblas_gemm_selector_pick(2, 96, 80, 512, b"t", b"n", 512, 512, 96, 1, C.byref(pick)) == 0
    assert pick.value == best.value
