"""Test helpers: seeded inputs, portBLAS-style comparisons, host<->device."""
import numpy as np

SEED = 20240917


def rng(tag: int = 0) -> np.random.Generator:
    return np.random.default_rng(SEED + tag)


def almost_equal(a, b, dtype=np.float32, mult=1.0):
    """portBLAS's scalar comparison (common/include/common/float_comparison.hpp:160-188):
    exact, both NaN, both inf, else absolute margin near zero and relative
    margin |a-b|/(|a|+|b|) otherwise (float 5e-3 / 1e-3, double 1e-10)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    rel = (5e-3 if np.dtype(dtype) == np.float32 else 1e-10) * mult
    absm = (1e-3 if np.dtype(dtype) == np.float32 else 1e-10) * mult
    eq = a == b
    both_nan = np.isnan(a) & np.isnan(b)
    both_inf = np.isinf(a) & np.isinf(b)
    with np.errstate(invalid="ignore", divide="ignore"):
        diff = np.abs(a - b)
        near0 = (a == 0) | (b == 0) | (diff < absm)
        ok_abs = diff < absm
        ok_rel = diff / (np.abs(a) + np.abs(b)) < rel
    return eq | both_nan | both_inf | np.where(near0, ok_abs, ok_rel)


def assert_almost_equal(a, b, dtype=np.float32, mult=1.0):
    ok = almost_equal(a, b, dtype, mult)
    if not np.all(ok):
        a = np.asarray(a).ravel()
        b = np.asarray(b).ravel()
        bad = np.flatnonzero(~np.asarray(ok).ravel())
        i = bad[0]
        raise AssertionError(f"{len(bad)} mismatches; first at {i}: {a[i]!r} vs {b[i]!r}")


def to_dev(a, torch, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def to_host(t):
    return t.detach().cpu().numpy()
