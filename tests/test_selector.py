"""Host-side checks of the tile-selector pieces (no GPU): the config table,
the feature vector, the size heuristic, and the FP64 oracle of the network
checked against finite differences (so it can in turn check the CUDA
kernels' gradients)."""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import mlp as omlp
from portblas_gb300 import _lib, build


@pytest.fixture(scope="module")
def L():
    build.build()
    return _lib.load()


def test_config_table(L):
    assert L.gbblas_sgemm_config_count() == 40
    assert L.gbblas_gemm_config_count() == 60
    seen = set()
    for c in range(60):
        v = [C.c_int() for _ in range(5)]
        assert L.gbblas_sgemm_config_info(c, *[C.byref(x) for x in v]) == 0
        method, tm, tn, split, raster = (x.value for x in v)
        assert method == (0 if c < 20 else (1 if c < 40 else 2))
        assert split in (1, 2, 4, 8, 16) and tm in (64, 128) and tn in (64, 128)
        seen.add((method, tm, tn, split, raster))
    assert len(seen) == 60
    assert L.gbblas_sgemm_config_info(60, None, None, None, None, None) == 1


@pytest.mark.parametrize("dtype,onehot", [(0, (1, 0)), (2, (0, 1))])
def test_features_match_definition(L, dtype, onehot):
    f = (C.c_float * 11)()
    assert L.gbblas_gemm_features(dtype, 1024, 3, 16384, b"t", b"N", 1030, 16, 1024, 64, C.addressof(f)) == 0
    got = np.frombuffer(f, dtype=np.float32)
    exp = [10 / 14, math.log2(3) / 14, 1.0, 1, 0, 6 / 16, 0, 0, 6 / 10, *onehot]
    np.testing.assert_allclose(got, exp, rtol=1e-6, atol=1e-7)
    g = (C.c_float * 11)()
    assert L.gbblas_sgemm_features(1024, 3, 16384, b"t", b"N", 1030, 16, 1024, 64, C.addressof(g)) == 0
    assert list(np.frombuffer(g, dtype=np.float32)[9:]) == [1.0, 0.0]
    assert L.gbblas_gemm_features(1, 8, 8, 8, b"n", b"n", 8, 8, 8, 1, C.addressof(f)) == 1  # BF16: no dense GEMM


def test_heuristic_tiers(L):
    h = L.gbblas_sgemm_heuristic_config
    assert h(100, 100, 100, 8) == 15
    assert h(200, 256, 10, 1) == 15
    assert h(1000, 10, 10, 1) == 5
    assert h(2048, 2048, 2048, 1) == 0
    assert h(8192, 100, 100, 1) == 20
    h64 = lambda m, n, k, b: L.gbblas_gemm_heuristic_config(2, m, n, k, b)
    assert h64(100, 100, 100, 8) == 55
    assert h64(1000, 10, 10, 1) == 45
    assert h64(8192, 100, 100, 1) == 40
    assert all(40 <= h64(m, m, m, 1) < 60 for m in (1, 300, 3000, 30000))


def test_mlp_oracle_gradient_finite_differences():
    g = np.random.default_rng(0)
    din, hid, dout, n = 5, 7, 4, 9
    count = hid * (din + 1) + 2 * hid * (hid + 1) + dout * (hid + 1)
    p = g.standard_normal(count) * 0.5
    x = g.standard_normal((n, din))
    t = g.standard_normal((n, dout))
    mask = (g.random((n, dout)) < 0.8).astype(float)
    valid = mask.sum()
    loss, grad = omlp.loss_grad(p, x, t, mask, din, hid, dout, valid)
    eps = 1e-6
    for i in g.choice(count, 25, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (omlp.loss_grad(pp, x, t, mask, din, hid, dout, valid)[0] -
              omlp.loss_grad(pm, x, t, mask, din, hid, dout, valid)[0]) / (2 * eps)
        assert abs(fd - grad[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, grad[i])


def test_selector_weight_file_format(tmp_path, L):
    from portblas_gb300.tuning import train
    p = train.init_params(3)
    path = tmp_path / "w.bin"
    train.write_bin(str(path), p)
    assert L.gbblas_sgemm_load_selector(str(path).encode()) == 0
    cfg = C.c_int()
    assert L.gbblas_sgemm_selector_pick(512, 512, 512, b"n", b"n", 512, 512, 512, 1, C.byref(cfg)) == 0
    assert 0 <= cfg.value < 40
    # the pick is always one of the element type's configs
    for m in (1, 77, 512, 5000):
        assert L.gbblas_gemm_selector_pick(0, m, m, m, b"n", b"t", m, m, m, 3, C.byref(cfg)) == 0
        assert 0 <= cfg.value < 40
        assert L.gbblas_gemm_selector_pick(2, m, m, m, b"n", b"t", m, m, m, 3, C.byref(cfg)) == 0
        assert 40 <= cfg.value < 60
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"nope")
    assert L.gbblas_sgemm_load_selector(str(bad).encode()) == 1
    # the shipped weights load again for the tests that follow
    shipped = __import__("os").path.join(__import__("os").path.dirname(build.LIB_PATH), "..", "tuning",
                                         "gemm_selector.bin")
    assert L.gbblas_sgemm_load_selector(shipped.encode()) == 0


def test_selector_picks_are_remembered_and_reset_by_new_weights(tmp_path, L):
    """AUTO remembers the network's pick per shape; loading new weights
    forgets it.  Two weight files whose output layer makes config 7, then
    config 23, the fastest for every input: the same shape picks 7, then 23."""
    from portblas_gb300.tuning import train
    cfg = C.c_int()
    paths = []
    for winner in (7, 23):
        p = train.init_params(5)
        out = train.OUT
        p[-(out * train.HID + out):] = 0.0  # last layer: weights and biases
        p[-out + winner] = -100.0           # predicted log-time: lowest wins
        path = tmp_path / f"w{winner}.bin"
        train.write_bin(str(path), p)
        paths.append(path)
    try:
        assert L.gbblas_sgemm_load_selector(str(paths[0]).encode()) == 0
        for _ in range(2):
            assert L.gbblas_sgemm_selector_pick(700, 300, 900, b"n", b"t", 704, 304, 700, 1, C.byref(cfg)) == 0
            assert cfg.value == 7
        assert L.gbblas_sgemm_load_selector(str(paths[1]).encode()) == 0
        assert L.gbblas_sgemm_selector_pick(700, 300, 900, b"n", b"t", 704, 304, 700, 1, C.byref(cfg)) == 0
        assert cfg.value == 23
    finally:
        shipped = __import__("os").path.join(__import__("os").path.dirname(build.LIB_PATH), "..", "tuning",
                                             "gemm_selector.bin")
        assert L.gbblas_sgemm_load_selector(shipped.encode()) == 0
