"""Host-side tile choice of the fixed split-BF16 SGEMM modes (no GPU
needed): which shapes run on 256 x 256 CTA-pair tiles, which on 256 x 128
CTA-pair tiles (x3 only), and which on one-CTA 128 x 128 / 128 x 64 tiles
with split-K.  The launcher takes its route from the same function, so these
cases pin what the GPU runs."""
import os
import subprocess
import sys

import pytest

from portblas_gb300 import blas, build

X3, X6 = blas.sgemm_mode_t.split_bf16x3, blas.sgemm_mode_t.split_bf16x6


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


# (m, n, k, batch) -> (x3 route, x6 route) on 152 SMs (76 CTA pairs)
ROUTES = [
    # square sizes where the pair tiles measured faster than 128 x 128 tiles
    ((2048, 2048, 2048, 1), (256, 256, 1), (256, 256, 1)),
    ((2304, 2304, 2304, 1), (256, 256, 1), (256, 256, 1)),
    ((2560, 2560, 2560, 1), (256, 256, 1), (256, 256, 1)),
    ((8192, 8192, 8192, 1), (256, 256, 1), (256, 256, 1)),
    # shallow K: the 256 x 256 tiles still fill the pairs
    ((8192, 8192, 128, 1), (256, 256, 1), (256, 256, 1)),
    ((2000, 1500, 300, 1), (256, 256, 1), (256, 256, 1)),
    ((512, 512, 512, 16), (256, 256, 1), (256, 256, 1)),
    ((1000, 1000, 300, 40), (256, 256, 1), (256, 256, 1)),
    # strided batches whose 256 x 256 tiles would be a quarter to two thirds
    # padding (measured 7-9% slower on them)
    ((384, 384, 384, 32), (128, 128, 1), (128, 128, 1)),
    ((300, 300, 300, 50), (256, 128, 1), (128, 128, 1)),
    # N below 256: two waves of 128 x 128 tiles take 256 x 128 pairs in x3
    ((1000, 200, 300, 20), (256, 128, 1), (128, 128, 1)),
    # too few tiles for half the pairs: 128 x 64 tiles, split-K when those
    # leave half the SMs idle
    ((1024, 1024, 1024, 1), (128, 64, 1), (128, 64, 1)),
    ((512, 512, 4096, 1), (128, 64, 4), (128, 64, 4)),
    # N at most 64 keeps 128 x 128 tiles (the 64-wide tile gains nothing)
    ((64, 64, 100000, 1), (128, 128, 1), (128, 128, 1)),
    ((100, 32, 64, 1), (128, 128, 1), (128, 128, 1)),
]


@pytest.mark.parametrize("shape,x3,x6", ROUTES, ids=["x".join(map(str, s)) for s, _, _ in ROUTES])
def test_routes_on_152_sms(shape, x3, x6):
    assert blas.sgemm_split_route(*shape, mode=X3) == x3
    assert blas.sgemm_split_route(*shape, mode=X6) == x6


def test_route_depends_on_sm_count():
    # 16 pair tiles leave most of 76 pairs idle, but fill 4 pairs exactly
    assert blas.sgemm_split_route(1024, 1024, 1024, 1, mode=X3, sm_count=152) == (128, 64, 1)
    assert blas.sgemm_split_route(1024, 1024, 1024, 1, mode=X3, sm_count=8) == (256, 256, 1)


def test_split_k_is_capped_by_depth_and_sixteen():
    # one 128 x 64 tile: split = min(152, k-blocks / 4, 16)
    tm, tn, ks = blas.sgemm_split_route(100, 64, 1 << 20, 1, mode=X3)
    assert (tm, ks) == (128, 1)  # n <= 64 keeps 128 x 128 tiles, no split
    assert blas.sgemm_split_route(100, 65, 1 << 20, 1, mode=X3) == (128, 64, 16)
    tm, tn, ks = blas.sgemm_split_route(100, 65, 512, 1, mode=X3)
    assert (tm, tn) == (128, 64) and 1 <= ks <= 16


def test_invalid_arguments():
    with pytest.raises(blas.InvalidArgument):
        blas.sgemm_split_route(-1, 8, 8)
    with pytest.raises(blas.InvalidArgument):
        blas.sgemm_split_route(8, 8, 8, mode=blas.sgemm_mode_t.auto)
    with pytest.raises(blas.InvalidArgument):
        blas.sgemm_split_route(8, 8, 8, sm_count=0)
    with pytest.raises(blas.UnsupportedException):
        blas.sgemm_split_route(1 << 31, 8, 8)


def test_pair_tiles_off_in_a_child_process():
    """GBBLAS_PAIR_TILES=0 (read once per process) sends every shape to the
    one-CTA tiles."""
    code = ("from portblas_gb300 import blas; M = blas.sgemm_mode_t; "
            "print(blas.sgemm_split_route(2048, 2048, 2048, 1, mode=M.split_bf16x3), "
            "blas.sgemm_split_route(300, 300, 300, 50, mode=M.split_bf16x3), "
            "blas.sgemm_split_route(2048, 2048, 2048, 1, mode=M.split_bf16x6))")
    here = os.path.dirname(os.path.abspath(__file__))
    env = dict(os.environ, GBBLAS_PAIR_TILES="0")
    r = subprocess.run([sys.executable, "-c", code], env=env, cwd=os.path.dirname(here), capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    assert r.stdout.split() == ["(128,", "128,", "1)"] * 3
