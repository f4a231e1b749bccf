"""Failure detection without a GPU fault: a device-side wait that nothing
will complete gives up after its wall-clock limit, records an error code in
the handle's device error word and returns; the host reads it as
GBBLAS_STATUS_TIMEOUT and the context stays usable."""
import numpy as np
import pytest

from tests.util import rng

pytestmark = pytest.mark.gpu

TIMEOUT = 4  # GBBLAS_STATUS_TIMEOUT


def test_bounded_wait_reports_timeout_and_context_survives(sb, torch_cuda):
    torch = torch_cuda
    from portblas_gb300 import _lib, blas
    L = _lib.load()
    assert L.gbblas_check_device_error(sb.handle) == 0  # start clean
    assert L.gbblas_selftest_wait_timeout(sb.handle, 5_000_000) == 0  # 5 ms limit
    assert L.gbblas_check_device_error(sb.handle) == TIMEOUT
    assert b"code 901" in L.gbblas_last_error()
    assert L.gbblas_check_device_error(sb.handle) == 0  # the word was cleared
    # the context still runs kernels correctly
    x = rng(3).uniform(-1, 1, 1 << 20).astype(np.float32)
    got = blas._asum(sb, x.size, torch.from_numpy(x).cuda(), 1)
    np.testing.assert_allclose(got, np.abs(x.astype(np.float64)).sum(), rtol=1e-6)
    with pytest.raises(blas.GbblasError):
        L.gbblas_selftest_wait_timeout(sb.handle, 1_000_000)
        sb.check_device_error()
