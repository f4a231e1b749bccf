"""Host-side tile schedule of the tcgen05 grouped GEMM (no GPU needed): which
problems get their K cut into slices (split-K) and how many tiles the
persistent kernel hands out.  The schedule is list scheduling, longest tile
first; split-K is chosen only where one problem's tiles would set the
makespan."""
import numpy as np
import pytest

from portblas_gb300 import blas, build
from tests.util import rng


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _p(m, n, k, alpha=1.0, ta="n", tb="n"):
    return dict(transa=ta, transb=tb, m=m, n=n, k=k, alpha=alpha)


def _out_tiles(p):
    return -(-p["m"] // 128) * -(-p["n"] // 128)


@pytest.mark.parametrize("dtype,bk", [("float32", 32), ("bfloat16", 64)])
def test_tall_skinny_is_split(dtype, bk):
    tiles, splits = blas.grouped_schedule([_p(48, 48, 1 << 18)], dtype=dtype)
    assert 1 < splits[0] <= 152 and tiles == splits[0]
    # every slice is at least 256 deep
    assert (1 << 18) / splits[0] >= 256


@pytest.mark.parametrize("dtype", ["float32", "bfloat16"])
def test_every_problem_keeps_its_tiles(dtype):
    """alpha == 0 (K treated as empty), m or n == 0 (no tiles), short and long
    K mixed: tiles = sum over problems of output tiles x slices."""
    probs = [_p(26, 165, 360, alpha=0.0), _p(0, 10, 10), _p(10, 0, 10), _p(300, 200, 0),
             _p(48, 48, 200000), _p(130, 300, 9001, ta="t"), _p(1, 1, 1), _p(37, 17, 510, tb="t")]
    tiles, splits = blas.grouped_schedule(probs, dtype=dtype)
    assert splits[1] == 0 and splits[2] == 0
    assert splits[0] == 1 and splits[3] == 1 and splits[6] == 1
    assert all(s >= 1 for i, s in enumerate(splits) if i not in (1, 2))
    assert splits[4] > 1
    assert tiles == sum(_out_tiles(p) * s for p, s in zip(probs, splits))


def test_many_short_problems_are_not_split():
    """The uneven batching workload (2048 problems, sizes log-uniform in
    [16, 512]): no tile dominates the load, so nothing is split."""
    g = rng(4)
    probs = []
    for _ in range(2048):
        m, n, k = (int(round(np.exp(g.uniform(np.log(16), np.log(512))))) for _ in range(3))
        probs.append(_p(m, n, k))
    for dtype in ("float32", "bfloat16"):
        tiles, splits = blas.grouped_schedule(probs, dtype=dtype)
        assert set(splits) == {1}
        assert tiles == sum(_out_tiles(p) for p in probs)


def test_one_large_problem_is_not_split():
    tiles, splits = blas.grouped_schedule([_p(4096, 4096, 4096)])
    assert splits == [1] and tiles == 32 * 32


def test_fewer_sms_split_less():
    probs = [_p(128, 128, 65536)] * 4
    t_big, s_big = blas.grouped_schedule(probs, sm_count=152)
    t_small, s_small = blas.grouped_schedule(probs, sm_count=8)
    assert s_big[0] > s_small[0] >= 1
    assert t_small <= 4 * 64


def test_schedule_argument_errors():
    with pytest.raises(blas.InvalidArgument):
        blas.grouped_schedule([_p(4, 4, 4)], sm_count=0)
    with pytest.raises(blas.InvalidArgument):
        blas.grouped_schedule([_p(4, 4, 4, ta="x")])
    with pytest.raises(blas.UnsupportedException):
        blas.grouped_schedule([_p(4, 4, 4)], dtype="float64")


def test_splitk_switch_off_and_forced(monkeypatch):
    """GBBLAS_GROUPED_SPLITK=0 never splits; =N cuts every problem of at
    least N k-blocks into N slices (capped at 256); short problems keep one."""
    probs = [_p(48, 48, 1 << 18), _p(128, 128, 4096), _p(16, 16, 64)]
    monkeypatch.setenv("GBBLAS_GROUPED_SPLITK", "0")
    tiles, splits = blas.grouped_schedule(probs, dtype="bfloat16")
    assert splits == [1, 1, 1] and tiles == 3
    monkeypatch.setenv("GBBLAS_GROUPED_SPLITK", "8")
    tiles, splits = blas.grouped_schedule(probs, dtype="bfloat16")  # k-blocks of 64: 4096, 64, 1
    assert splits == [8, 8, 1] and tiles == 17
    monkeypatch.setenv("GBBLAS_GROUPED_SPLITK", "1000")
    _, splits = blas.grouped_schedule(probs, dtype="float32")  # k-blocks of 32: 8192, 128, 2
    assert splits == [256, 1, 1]
