"""GPU parity of asum / nrm2 / dot / iamax / iamin against the oracle,
through the C ABI (portblas_gb300.blas), on portBLAS's test sweeps
(test/unittest/blas1/blas1_{asum,nrm2,dot,iamax,iamin}_test.cpp)."""
import json
import os

import numpy as np
import pytest

import oracle
from tests.util import rng, to_dev, to_host, assert_almost_equal

pytestmark = pytest.mark.gpu
KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kat.json")))


def _vec(g, n, inc, dtype=np.float32):
    # fill_random's range [-2, 5] (test/blas_test.hpp:107-140)
    return g.uniform(-2, 5, max(1, n * abs(inc))).astype(dtype)


@pytest.mark.parametrize("api", ["async", "sync"])
@pytest.mark.parametrize("n", [11, 65, 10000, 1002400])
@pytest.mark.parametrize("inc", [1, 4, -1, -3])
def test_asum(sb, torch_cuda, api, n, inc):
    torch = torch_cuda
    from portblas_gb300 import blas
    x = _vec(rng(n + inc), n, inc) / (n * abs(inc))  # blas1_asum_test.cpp:46-49
    xd = to_dev(x, torch)
    ref = oracle.asum(n, x, inc)
    if api == "async":
        rs = torch.zeros(1, device="cuda")
        blas._asum(sb, n, xd, inc, rs)
        got = float(to_host(rs)[0])
    else:
        got = blas._asum(sb, n, xd, inc)
    assert_almost_equal(got, ref)
    assert abs(got - ref) <= 4e-7 * abs(ref) + 1e-30  # compensated: near FP32 rounding of the true sum


@pytest.mark.parametrize("api", ["async", "sync"])
@pytest.mark.parametrize("n", [11, 1002, 1002400])
@pytest.mark.parametrize("inc", [1, 4, -3])
def test_nrm2(sb, torch_cuda, api, n, inc):
    torch = torch_cuda
    from portblas_gb300 import blas
    x = _vec(rng(2 * n + inc), n, inc)
    xd = to_dev(x, torch)
    ref = oracle.nrm2(n, x, inc)
    if api == "async":
        rs = torch.zeros(1, device="cuda")
        blas._nrm2(sb, n, xd, inc, rs)
        got = float(to_host(rs)[0])
    else:
        got = blas._nrm2(sb, n, xd, inc)
    assert_almost_equal(got, ref)
    assert abs(got - ref) <= 4e-7 * ref


@pytest.mark.parametrize("scale", [1e30, 1e-30, 1e-42])
def test_nrm2_scaling_no_overflow(sb, torch_cuda, scale):
    torch = torch_cuda
    from portblas_gb300 import blas
    x = (rng(7).standard_normal(4097) * scale).astype(np.float32)
    got = blas._nrm2(sb, len(x), to_dev(x, torch), 1)
    ref = oracle.nrm2(len(x), x, 1)
    assert np.isfinite(got) and ref > 0
    assert abs(got - ref) <= 1e-6 * ref + 1e-45


@pytest.mark.parametrize("api", ["async", "sync"])
@pytest.mark.parametrize("n", [11, 65, 1002, 1002400])
@pytest.mark.parametrize("incx,incy", [(1, 1), (4, 3), (1, 3), (-2, 1)])
def test_dot(sb, torch_cuda, api, n, incx, incy):
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(3 * n + incx)
    x, y = _vec(g, n, incx), _vec(g, n, incy)
    ref = oracle.dot(n, x, incx, y, incy)
    xd, yd = to_dev(x, torch), to_dev(y, torch)
    if api == "async":
        rs = torch.zeros(1, device="cuda")
        blas._dot(sb, n, xd, incx, yd, incy, rs)
        got = float(to_host(rs)[0])
    else:
        got = blas._dot(sb, n, xd, incx, yd, incy)
    assert_almost_equal(got, ref)
    assert abs(got - ref) <= 4e-7 * abs(ref) + 1e-6


def test_dot_n0_leaves_result(sb, torch_cuda):
    torch = torch_cuda
    from portblas_gb300 import blas
    rs = torch.full((1,), 42.0, device="cuda")
    x = torch.ones(4, device="cuda")
    blas._dot(sb, 0, x, 1, x, 1, rs)
    sb.wait()
    assert float(rs.item()) == 42.0


def _iam_input(case):
    size, inc = case["n"], case["incx"]
    length = size * abs(inc)
    if case["mode"] == "limit":
        return np.full(length, case["fill"], dtype=np.float32)
    if case["mode"] == "incrementing":
        return np.arange(length, dtype=np.float32)
    return (length - 1 - np.arange(length)).astype(np.float32)


@pytest.mark.parametrize("case", KAT["iaminmax"], ids=lambda c: f"{c['op']}-{c['mode']}-{c['n']}-{c['incx']}")
def test_iaminmax_kat(sb, torch_cuda, case):
    torch = torch_cuda
    from portblas_gb300 import blas
    x = to_dev(_iam_input(case), torch)
    fn = blas._iamax if case["op"] == "iamax" else blas._iamin
    assert fn(sb, case["n"], x, case["incx"]) == case["expected"]
    rs = torch.full((1,), -5, dtype=torch.int32, device="cuda")
    fn(sb, case["n"], x, case["incx"], rs)
    assert int(rs.item()) == case["expected"]


@pytest.mark.parametrize("n", [11, 65, 1000000, 1 << 22])
@pytest.mark.parametrize("inc", [1, 5])
@pytest.mark.parametrize("op", ["iamax", "iamin"])
def test_iaminmax_random_bitexact(sb, torch_cuda, n, inc, op):
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(n + inc + (op == "iamin"))
    x = _vec(g, n, inc)
    # plant ties of the extreme |x| at several random logical indices
    idx = g.choice(n, size=min(8, n), replace=False)
    if op == "iamax":
        v = np.float32(8 * np.abs(x).max())
    else:
        v = np.float32(0.5 * np.abs(x[: n * inc: inc]).min())
    x[idx * inc] = v * g.choice([-1, 1], size=len(idx)).astype(np.float32)
    exp = (oracle.iamax if op == "iamax" else oracle.iamin)(n, x, inc)
    assert exp == int(idx.min())
    fn = blas._iamax if op == "iamax" else blas._iamin
    assert fn(sb, n, to_dev(x, torch), inc) == exp


def test_iamax_nan_and_empty(sb, torch_cuda):
    torch = torch_cuda
    from portblas_gb300 import blas
    x = to_dev(np.array([np.nan, 1.0, -3.0, np.nan, 3.0], dtype=np.float32), torch)
    assert blas._iamax(sb, 5, x, 1) == 2
    assert blas._iamin(sb, 5, x, 1) == 1
    assert blas._iamax(sb, 0, x, 1) == 2**31 - 1
    assert blas._iamax(sb, 5, x, -1) == 0


@pytest.mark.parametrize("case", KAT["blas1"], ids=lambda c: f"{c['op']}-{c['n']}-{c['incx']}")
def test_blas1_kat(sb, torch_cuda, case):
    torch = torch_cuda
    from portblas_gb300 import blas
    x = to_dev(np.array(case["x"], dtype=np.float32), torch)
    op = case["op"]
    if op == "dot":
        got = blas._dot(sb, case["n"], x, case["incx"], to_dev(np.array(case["y"], dtype=np.float32), torch),
                        case["incy"])
    else:
        got = getattr(blas, "_" + op)(sb, case["n"], x, case["incx"])
    assert got == pytest.approx(case["expected"], rel=1e-6)


@pytest.mark.parametrize("n", [1 << 26])
def test_full_size_properties(sb, torch_cuda, n):
    """Config-sized (2^26) checks by properties: asum(x) == asum(-x) exactly
    and equals a concatenation checksum; dot(x, x) == nrm2(x)^2; determinism."""
    torch = torch_cuda
    from portblas_gb300 import blas
    gen = torch.Generator(device="cuda").manual_seed(11)
    x = torch.randn(n, device="cuda", generator=gen)
    a1 = blas._asum(sb, n, x, 1)
    a2 = blas._asum(sb, n, -x, 1)
    assert a1 == a2
    assert blas._asum(sb, n, x, 1) == a1  # deterministic
    h = n // 2
    parts = blas._asum(sb, h, x[:h], 1) + blas._asum(sb, n - h, x[h:], 1)
    assert abs(parts - a1) <= 1e-6 * a1
    nr = blas._nrm2(sb, n, x, 1)
    dd = blas._dot(sb, n, x, 1, x, 1)
    assert abs(dd - nr * nr) <= 2e-6 * dd
    ref = float(torch.linalg.vector_norm(x.double()).item())
    assert abs(nr - ref) <= 1e-6 * ref


def test_blas1_chain_in_captured_cuda_graph(torch_cuda):
    """Full-wave BLAS-1 reductions (launched with programmatic dependent
    launch) captured back to back into a CUDA graph and replayed twice: the
    programmatic edges keep stream order, so every result matches the
    oracle, and a replay after changing x sees the new x."""
    torch = torch_cuda
    from portblas_gb300 import blas, build
    build.build()
    n = 1 << 23  # a full wave of CTAs
    g = rng(97)
    x = g.standard_normal(n).astype(np.float32)
    y = g.standard_normal(n).astype(np.float32)
    s = torch.cuda.Stream()
    h = blas.SB_Handle(s)
    xd, yd = to_dev(x, torch), to_dev(y, torch)
    out = torch.zeros(4, device="cuda")
    idx = torch.zeros(2, dtype=torch.int32, device="cuda")

    def chain():
        blas._asum(h, n, xd, 1, out[0:1])
        blas._nrm2(h, n, xd, 1, out[1:2])
        blas._dot(h, n, xd, 1, yd, 1, out[2:3])
        blas._iamax(h, n, xd, 1, idx[0:1])
        blas._iamin(h, n, xd, 1, idx[1:2])
        blas._asum(h, n, yd, 1, out[3:4])

    with torch.cuda.stream(s):
        chain()  # temp memory and kernel attributes set up outside the capture
    s.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        chain()
    for it in range(2):
        if it == 1:
            x = (x * -0.5).astype(np.float32)
            xd.copy_(torch.from_numpy(x).cuda())
        out.zero_()
        idx.zero_()
        torch.cuda.synchronize()
        graph.replay()
        torch.cuda.synchronize()
        o = to_host(out)
        i = to_host(idx)
        assert abs(o[0] - oracle.asum(n, x, 1)) <= 1e-6 * oracle.asum(n, x, 1)
        assert abs(o[1] - oracle.nrm2(n, x, 1)) <= 1e-6 * oracle.nrm2(n, x, 1)
        d = oracle.dot(n, x, 1, y, 1)
        assert abs(o[2] - d) <= 1e-6 * float(np.abs(x.astype(np.float64) * y).sum())
        assert int(i[0]) == oracle.iamax(n, x, 1) and int(i[1]) == oracle.iamin(n, x, 1)
        assert abs(o[3] - oracle.asum(n, y, 1)) <= 1e-6 * oracle.asum(n, y, 1)
    h.close()
