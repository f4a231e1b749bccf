"""GPU parity of extension::_reduction against the oracle through the C ABI,
on portBLAS's sweep (test/unittest/extension/reduction_test.cpp:43-241)."""
import json
import os

import numpy as np
import pytest

import oracle
from tests.util import rng, to_dev, to_host, assert_almost_equal

pytestmark = pytest.mark.gpu
KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kat.json")))
OPS = ["add", "product", "max", "min", "abs_add", "mean"]


def _op_class(op):
    from portblas_gb300 import blas
    return {"add": blas.AddOperator, "product": blas.ProductOperator, "max": blas.MaxOperator,
            "min": blas.MinOperator, "abs_add": blas.AbsoluteAddOperator, "mean": blas.MeanOperator}[op]


def _run(sb, torch, op, dim, data, ld, rows, cols, dtype=np.float32):
    from portblas_gb300 import blas
    nout = cols if dim == "inner" else rows
    out = torch.full((nout,), 7.0, dtype=torch.float32 if dtype == np.float32 else torch.float64, device="cuda")
    rd = blas.reduction_dim_t.inner if dim == "inner" else blas.reduction_dim_t.outer
    blas.extension._reduction(_op_class(op), sb, to_dev(data.astype(dtype), torch), ld, out, rows, cols, rd)
    return to_host(out)


@pytest.mark.parametrize("case", KAT["reduction"], ids=lambda c: f"{c['op']}-{c['dim']}-ld{c['ld']}")
def test_reduction_kat(sb, torch_cuda, case):
    got = _run(sb, torch_cuda, case["op"], case["dim"], np.array(case["data"]), case["ld"], case["rows"],
               case["cols"])
    np.testing.assert_array_equal(got, np.array(case["expected"], dtype=np.float32))


@pytest.mark.parametrize("rows", [1, 7, 513])
@pytest.mark.parametrize("cols", [1, 15, 1000, 1337, 8195])
@pytest.mark.parametrize("ld_mul", [1, 2, 3])
@pytest.mark.parametrize("op", OPS)
@pytest.mark.parametrize("dim", ["inner", "outer"])
def test_reduction_sweep(sb, torch_cuda, rows, cols, ld_mul, op, dim):
    g = rng(rows * 7 + cols + ld_mul)
    ld = rows * ld_mul
    lo, hi = (-2.0, 1.0) if op == "product" else (-2.0, 5.0)
    data = g.uniform(lo, hi, ld * cols).astype(np.float32)
    ref = oracle.reduction(op, dim, data, ld, rows, cols)
    got = _run(sb, torch_cuda, op, dim, data, ld, rows, cols)
    if op in ("max", "min"):
        np.testing.assert_array_equal(got, ref.astype(np.float32))
    elif op == "product":
        assert_almost_equal(got, ref.astype(np.float32))
    else:
        assert_almost_equal(got, ref)
        np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-6 * np.abs(ref).max())


@pytest.mark.parametrize("dim", ["inner", "outer"])
@pytest.mark.parametrize("rows,cols", [(100000, 3), (3, 100000), (4096 * 5 + 3, 17)])
def test_reduction_split_shapes(sb, torch_cuda, dim, rows, cols):
    g = rng(rows + cols)
    data = g.standard_normal(rows * cols).astype(np.float32)
    for op in ("add", "mean", "max"):
        ref = oracle.reduction(op, dim, data, rows, rows, cols)
        got = _run(sb, torch_cuda, op, dim, data, rows, rows, cols)
        if op == "max":
            np.testing.assert_array_equal(got, ref.astype(np.float32))
        else:
            np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5)


def test_reduction_double(sb, torch_cuda):
    g = rng(99)
    data = g.uniform(-2, 5, 513 * 1000)
    for dim in ("inner", "outer"):
        ref = oracle.reduction("add", dim, data, 513, 513, 1000, dtype=np.float64)
        got = _run(sb, torch_cuda, "add", dim, data, 513, 513, 1000, dtype=np.float64)
        assert_almost_equal(got, ref, dtype=np.float64)


@pytest.mark.parametrize("dim", ["inner", "outer"])
def test_reduction_full_size(sb, torch_cuda, dim):
    """16384 x 16384 (the benchmark size) checked with torch FP64 sums and the
    sum-of-sums identity inner.sum() == outer.sum()."""
    torch = torch_cuda
    from portblas_gb300 import blas
    n = 16384
    gen = torch.Generator(device="cuda").manual_seed(3)
    a = torch.rand(n * n, device="cuda", generator=gen) * 2 - 1
    out = torch.empty(n, device="cuda")
    rd = blas.reduction_dim_t.inner if dim == "inner" else blas.reduction_dim_t.outer
    blas.extension._reduction(blas.AddOperator, sb, a, n, out, n, n, rd)
    A = a.view(n, n)  # row r of this view is column r of the column-major matrix
    ref = A.double().sum(1) if dim == "inner" else A.double().sum(0)
    err = (out.double() - ref).abs().max().item()
    assert err <= 1e-5 * 128


@pytest.mark.parametrize("op", OPS)
@pytest.mark.parametrize("dim", ["inner", "outer"])
@pytest.mark.parametrize("rows,cols,ld", [(1000, 700, 1000), (4100, 300, 4104), (520, 1030, 520),
                                          (130, 5000, 132), (9000, 64, 9000)])
def test_reduction_tma_stream_path(sb, torch_cuda, op, dim, rows, cols, ld):
    """Shapes whose ld satisfies the tensor-map rules take the TMA-fed sweeps;
    ragged tiles must not leak zero fill into Max / Min / Product."""
    g = rng(rows * 3 + cols + ld)
    lo, hi = (0.995, 1.005) if op == "product" else (-5.0, -1.0)  # all-negative data catches a zero leak in Max
    if op == "min":
        lo, hi = 1.0, 5.0  # all-positive data catches a zero leak in Min
    data = g.uniform(lo, hi, ld * cols).astype(np.float32)
    ref = oracle.reduction(op, dim, data, ld, rows, cols)
    got = _run(sb, torch_cuda, op, dim, data, ld, rows, cols)
    if op in ("max", "min"):
        np.testing.assert_array_equal(got, ref.astype(np.float32))
    elif op == "product":
        np.testing.assert_allclose(got, ref, rtol=1e-3)
    else:
        np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-6 * np.abs(ref).max())
