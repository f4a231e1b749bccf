"""Grouped GEMM over uneven problems (persistent kernel, device tile
scheduler, CUDA-graph replay): each problem checked against the oracle with
blas::_gemm semantics."""
import numpy as np
import pytest

import oracle
from tests.util import rng, assert_almost_equal

pytestmark = pytest.mark.gpu


def _problems(torch, g, count, lo, hi, dtype):
    probs, host = [], []
    for i in range(count):
        m, n, k = (int(round(np.exp(g.uniform(np.log(lo), np.log(hi))))) for _ in range(3))
        ta, tb = bool(g.integers(2)), bool(g.integers(2))
        alpha = float(g.choice([1.0, 1.5, 0.0]))
        beta = float(g.choice([0.0, 0.5]))
        lda, ldb, ldc = (k if ta else m) + int(g.integers(3)), (n if tb else k) + int(g.integers(3)), m + 1
        a = g.uniform(-1, 1, lda * (m if ta else k)).astype(np.float32)
        b = g.uniform(-1, 1, ldb * (k if tb else n)).astype(np.float32)
        c = g.uniform(-1, 1, ldc * n).astype(np.float32)
        if dtype == "bfloat16":  # the oracle sees exactly the BF16 values
            a = torch.from_numpy(a).bfloat16().float().numpy()
            b = torch.from_numpy(b).bfloat16().float().numpy()
        tdt = torch.bfloat16 if dtype == "bfloat16" else torch.float32
        ad, bd = torch.from_numpy(a).to(tdt).cuda(), torch.from_numpy(b).to(tdt).cuda()
        cd = torch.from_numpy(c).cuda()
        probs.append(dict(transa="t" if ta else "n", transb="t" if tb else "n", m=m, n=n, k=k, alpha=alpha, a=ad,
                          lda=lda, b=bd, ldb=ldb, beta=beta, c=cd, ldc=ldc))
        host.append((ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc))
    return probs, host


def _check(probs, host):
    for p, (ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc) in zip(probs, host):
        ref = oracle.gemm(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc)
        got = p["c"].cpu().numpy().reshape(n, ldc).T[:m]
        assert_almost_equal(got, ref)
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5 * max(1, k))


METHODS = ["tcgen05", "simt"]


@pytest.fixture
def method(request, monkeypatch):
    monkeypatch.setenv("GBBLAS_GROUPED_METHOD", request.param)
    return request.param


@pytest.mark.parametrize("method", METHODS, indirect=True)
@pytest.mark.parametrize("dtype", ["float32", "bfloat16"])
def test_grouped_one_shot(sb, torch_cuda, dtype, method):
    from portblas_gb300 import blas
    probs, host = _problems(torch_cuda, rng(31), 64, 1, 300, dtype)
    blas._gemm_grouped(sb, probs, dtype=dtype)
    _check(probs, host)
    sb.check_device_error()


@pytest.mark.parametrize("method", METHODS, indirect=True)
def test_grouped_long_k_accuracy(sb, torch_cuda, method):
    """K well past the accumulator promotion interval: FP32-level accuracy."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(43)
    probs, host = [], []
    for (m, n, k) in [(130, 70, 3000), (64, 200, 1100), (1, 1, 5000)]:
        a = (g.choice([-1.0, 1.0], m * k) * np.exp2(g.uniform(-8, 8, m * k))).astype(np.float32)
        b = (g.choice([-1.0, 1.0], k * n) * np.exp2(g.uniform(-8, 8, k * n))).astype(np.float32)
        c = np.zeros(m * n, np.float32)
        probs.append(dict(transa="n", transb="n", m=m, n=n, k=k, alpha=1.0, a=torch.from_numpy(a).cuda(), lda=m,
                          b=torch.from_numpy(b).cuda(), ldb=k, beta=0.0, c=torch.from_numpy(c).cuda(), ldc=m))
        host.append((m, n, k, a, b))
    blas._gemm_grouped(sb, probs, dtype="float32")
    for p, (m, n, k, a, b) in zip(probs, host):
        ref = oracle.gemm(False, False, m, n, k, 1.0, a, m, b, k, 0.0, None, m)
        scale = oracle.gemm_absscale(False, False, m, n, k, 1.0, a, m, b, k, 0.0, None, m)
        got = p["c"].cpu().numpy().reshape(n, m).T
        assert (np.abs(got - ref) / scale).max() <= 2.0 * (k + 4) * 2.0 ** -24


@pytest.mark.parametrize("method", METHODS, indirect=True)
@pytest.mark.parametrize("dtype", ["float32", "bfloat16"])
def test_grouped_plan_graph_replay(sb, torch_cuda, dtype, method):
    """The captured graph replays correctly, twice (scheduler counters reset)."""
    torch = torch_cuda
    from portblas_gb300 import blas
    probs, host = _problems(torch, rng(37), 40, 16, 512, dtype)
    c0 = [p["c"].clone() for p in probs]
    plan = blas.GroupedPlan(sb, probs, dtype=dtype)
    plan.run()
    sb.wait()
    _check(probs, host)
    for p, c in zip(probs, c0):
        p["c"].copy_(c)
    plan.run()
    sb.wait()
    _check(probs, host)
    plan.close()


def test_grouped_invalid(sb, torch_cuda):
    torch = torch_cuda
    from portblas_gb300 import blas
    x = torch.zeros(16, device="cuda")
    bad = [dict(transa="x", transb="n", m=4, n=4, k=4, alpha=1.0, a=x, lda=4, b=x, ldb=4, beta=0.0, c=x, ldc=4)]
    with pytest.raises(blas.InvalidArgument):
        blas._gemm_grouped(sb, bad)
    with pytest.raises(blas.UnsupportedException):
        blas._gemm_grouped(sb, [dict(bad[0], transa="n")], dtype="float64")


@pytest.mark.parametrize("method", ["tcgen05"], indirect=True)
@pytest.mark.parametrize("ta,tb", [(True, False), (False, True), (True, True), (False, False)])
def test_grouped_bf16_aligned_operands_read_in_place(sb, torch_cuda, method, ta, tb):
    """BF16 operands that are K-contiguous with a 16-byte-aligned leading
    dimension are mapped by TMA in place (no conversion pass); mixed with
    operands that need the pass, against the oracle."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(53 + 2 * ta + tb)
    probs, host = [], []
    for i in range(24):
        m, n, k = (int(g.integers(1, 300)) for _ in range(3))
        # K-contiguous operands get ld rounded up to 8 elements (16 bytes)
        lda = ((k + 7) // 8) * 8 if ta else m + int(g.integers(3))
        ldb = ((k + 7) // 8) * 8 if not tb else n + int(g.integers(3))
        ldc = m
        a = torch.from_numpy(g.uniform(-1, 1, lda * (m if ta else k)).astype(np.float32)).bfloat16()
        b = torch.from_numpy(g.uniform(-1, 1, ldb * (k if tb else n)).astype(np.float32)).bfloat16()
        c = np.zeros(ldc * n, np.float32)
        probs.append(dict(transa="t" if ta else "n", transb="t" if tb else "n", m=m, n=n, k=k, alpha=1.0,
                          a=a.cuda(), lda=lda, b=b.cuda(), ldb=ldb, beta=0.0, c=torch.from_numpy(c).cuda(), ldc=ldc))
        host.append((ta, tb, m, n, k, 1.0, a.float().numpy(), lda, b.float().numpy(), ldb, 0.0, c, ldc))
    blas._gemm_grouped(sb, probs, dtype="bfloat16")
    _check(probs, host)
    sb.check_device_error()


@pytest.mark.parametrize("method", METHODS, indirect=True)
@pytest.mark.parametrize("dtype", ["float32", "bfloat16"])
def test_grouped_large_problems_tile_grouping(sb, torch_cuda, dtype, method):
    """Problems with more than 8 tile rows (the scheduler walks a problem's
    tiles in groups of 8 rows), k not a multiple of the k-block, mixed with
    tiny ones; sampled entries against the oracle."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(61)
    shapes = [(1500, 700, 333, True, False), (1100, 1300, 97, False, True), (3, 5, 7, False, False),
              (1025, 129, 65, True, True)]
    probs, host = [], []
    for (m, n, k, ta, tb) in shapes:
        lda, ldb, ldc = (k if ta else m) + 1, (n if tb else k) + 3, m + 2
        a = g.uniform(-1, 1, lda * (m if ta else k)).astype(np.float32)
        b = g.uniform(-1, 1, ldb * (k if tb else n)).astype(np.float32)
        c = g.uniform(-1, 1, ldc * n).astype(np.float32)
        if dtype == "bfloat16":
            a = torch.from_numpy(a).bfloat16().float().numpy()
            b = torch.from_numpy(b).bfloat16().float().numpy()
        tdt = torch.bfloat16 if dtype == "bfloat16" else torch.float32
        probs.append(dict(transa="t" if ta else "n", transb="t" if tb else "n", m=m, n=n, k=k, alpha=1.25,
                          a=torch.from_numpy(a).to(tdt).cuda(), lda=lda, b=torch.from_numpy(b).to(tdt).cuda(),
                          ldb=ldb, beta=0.5, c=torch.from_numpy(c).cuda(), ldc=ldc))
        host.append((ta, tb, m, n, k, a, lda, b, ldb, c, ldc))
    blas._gemm_grouped(sb, probs, dtype=dtype)
    for p, (ta, tb, m, n, k, a, lda, b, ldb, c, ldc) in zip(probs, host):
        rows = g.integers(0, m, 64)
        cols = g.integers(0, n, 64)
        ref = oracle.gemm(ta, tb, m, n, k, 1.25, a, lda, b, ldb, 0.5, c, ldc, rows=rows, cols=cols)
        got = p["c"].cpu().numpy().reshape(n, ldc).T[rows, cols]
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5 * max(1, k))
    sb.check_device_error()


@pytest.mark.parametrize("method", ["tcgen05"], indirect=True)
@pytest.mark.parametrize("dtype", ["float32", "bfloat16"])
def test_grouped_split_k_long_k(sb, torch_cuda, dtype, method):
    """A few long-K problems beside a small one: the plan cuts their K into
    slices (split-K, tall-skinny); the FP32 partials of the slices are added
    up a fixed fold tree (children in index order, whichever CTA arrives
    last), so two runs agree bit for bit, and beta is applied once.  Sampled entries against the oracle,
    normalised by |alpha| |A||B| + |beta C|."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(71)
    shapes = [(48, 48, 1 << 17, False, False), (200, 130, 20000, True, False), (130, 300, 9001, False, True),
              (1, 1, 70000, True, True), (20, 30, 40, False, False)]
    probs, host = [], []
    for (m, n, k, ta, tb) in shapes:
        lda, ldb, ldc = (k if ta else m) + 1, (n if tb else k) + 2, m + 3
        a = g.uniform(-1, 1, lda * (m if ta else k)).astype(np.float32)
        b = g.uniform(-1, 1, ldb * (k if tb else n)).astype(np.float32)
        c = g.uniform(-1, 1, ldc * n).astype(np.float32)
        if dtype == "bfloat16":
            a = torch.from_numpy(a).bfloat16().float().numpy()
            b = torch.from_numpy(b).bfloat16().float().numpy()
        tdt = torch.bfloat16 if dtype == "bfloat16" else torch.float32
        probs.append(dict(transa="t" if ta else "n", transb="t" if tb else "n", m=m, n=n, k=k, alpha=1.5,
                          a=torch.from_numpy(a).to(tdt).cuda(), lda=lda, b=torch.from_numpy(b).to(tdt).cuda(),
                          ldb=ldb, beta=0.5, c=torch.from_numpy(c).cuda(), ldc=ldc))
        host.append((ta, tb, m, n, k, a, lda, b, ldb, c, ldc))
    c0 = [p["c"].clone() for p in probs]
    plan = blas.GroupedPlan(sb, probs, dtype=dtype)
    tiles, splits = plan.info()
    assert splits > 1 and tiles > 8
    plan.run()
    sb.wait()
    first = [p["c"].clone() for p in probs]
    for p, (ta, tb, m, n, k, a, lda, b, ldb, c, ldc) in zip(probs, host):
        rows = g.integers(0, m, 48)
        cols = g.integers(0, n, 48)
        ref = oracle.gemm(ta, tb, m, n, k, 1.5, a, lda, b, ldb, 0.5, c, ldc, rows=rows, cols=cols)
        scale = oracle.gemm_absscale(ta, tb, m, n, k, 1.5, a, lda, b, ldb, 0.5, c, ldc, rows=rows, cols=cols)
        got = p["c"].cpu().numpy().reshape(n, ldc).T[rows, cols]
        assert (np.abs(got - ref) / scale).max() <= 1e-5, (m, n, k)
    for p, c in zip(probs, c0):
        p["c"].copy_(c)
    plan.run()
    sb.wait()
    for p, f in zip(probs, first):
        assert torch.equal(p["c"], f)
    plan.close()
    sb.check_device_error()


@pytest.mark.parametrize("method", ["tcgen05"], indirect=True)
@pytest.mark.parametrize("ta,tb", [(False, True), (False, False), (True, True)])
def test_grouped_bf16_rows_contiguous_read_in_place(sb, torch_cuda, method, ta, tb):
    """BF16 operands whose rows are contiguous (A 'n', B 't') with a leading
    dimension that is a multiple of 8 elements and a 16-byte-aligned start
    are read in place as MN-major tiles (two 64-row boxes per tile): rows
    below, at and above 64 and 128 (second box partly or wholly outside),
    ragged K, views 8 elements (16 bytes) and 1 element into a buffer (the
    latter takes the conversion pass), a long-K problem cut into slices;
    every C entry against the oracle."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(700 + 2 * ta + tb)
    shapes = [(1, 1, 1), (8, 16, 5), (48, 48, 300), (64, 64, 64), (65, 130, 129), (128, 128, 200), (136, 72, 17),
              (200, 256, 70), (40, 24, 20000)]
    probs, host, keep = [], [], []
    for i, (m, n, k) in enumerate(shapes):
        shift = 8 if i % 3 == 1 else (1 if i % 3 == 2 and i < 8 else 0)
        lda = k + 1 if ta else ((m + 7) // 8) * 8 + 8 * (i % 2)
        ldb = ((n + 7) // 8) * 8 + 8 * ((i + 1) % 2) if tb else k + 3
        ldc = m + 2
        sa, sbs = lda * (m if ta else k), ldb * (k if tb else n)
        a = torch.from_numpy(g.uniform(-1, 1, sa).astype(np.float32)).bfloat16()
        b = torch.from_numpy(g.uniform(-1, 1, sbs).astype(np.float32)).bfloat16()
        abuf = torch.zeros(shift + sa, dtype=torch.bfloat16, device="cuda")
        bbuf = torch.zeros(shift + sbs, dtype=torch.bfloat16, device="cuda")
        abuf[shift:].copy_(a.cuda())
        bbuf[shift:].copy_(b.cuda())
        keep += [abuf, bbuf]
        c = g.uniform(-1, 1, ldc * n).astype(np.float32)
        probs.append(dict(transa="t" if ta else "n", transb="t" if tb else "n", m=m, n=n, k=k, alpha=1.25,
                          a=abuf[shift:], lda=lda, b=bbuf[shift:], ldb=ldb, beta=0.5,
                          c=torch.from_numpy(c).cuda(), ldc=ldc))
        host.append((ta, tb, m, n, k, 1.25, a.float().numpy(), lda, b.float().numpy(), ldb, 0.5, c, ldc))
    plan = blas.GroupedPlan(sb, probs, dtype="bfloat16")
    plan.run()
    sb.wait()
    _check(probs, host)
    plan.close()
    sb.check_device_error()


@pytest.mark.parametrize("method", ["tcgen05"], indirect=True)
@pytest.mark.parametrize("shift", [0, 1])
def test_grouped_bf16_operand_alignment(sb, torch_cuda, method, shift):
    """BF16 operands moved into the K-major tiles with 32-bit loads: views
    that start in the odd half of a 4-byte word (shift 1) or on a word
    (shift 0), each ending exactly at the end of its buffer, odd and even
    leading dimensions, both transposes, rows and K that are not multiples of
    the 64 x 64 (transposed) or 8-wide (K-contiguous) pieces: every C entry
    against the oracle."""
    torch = torch_cuda
    from portblas_gb300 import blas
    g = rng(500 + shift)
    shapes = [(1, 1, 1), (63, 65, 3), (64, 64, 64), (65, 127, 129), (130, 7, 300), (17, 200, 64), (2, 3, 9),
              (129, 66, 17)]
    probs, host, keep = [], [], []
    for i, (m, n, k) in enumerate(shapes):
        for ta in (False, True):
            tb = bool((i + ta) % 2)
            pa, pb = i % 3, (i + 1) % 2
            lda, ldb, ldc = (k if ta else m) + pa, (n if tb else k) + pb, m + 1
            sa, sbs = lda * ((m if ta else k) - 1) + (k if ta else m), ldb * ((k if tb else n) - 1) + (n if tb else k)
            a = torch.from_numpy(g.uniform(-1, 1, sa).astype(np.float32)).bfloat16()
            b = torch.from_numpy(g.uniform(-1, 1, sbs).astype(np.float32)).bfloat16()
            abuf = torch.empty(shift + sa, dtype=torch.bfloat16, device="cuda")
            bbuf = torch.empty(shift + sbs, dtype=torch.bfloat16, device="cuda")
            abuf[shift:].copy_(a.cuda())
            bbuf[shift:].copy_(b.cuda())
            c = g.uniform(-1, 1, ldc * n).astype(np.float32)
            keep += [abuf, bbuf]
            probs.append(dict(transa="t" if ta else "n", transb="t" if tb else "n", m=m, n=n, k=k, alpha=1.0,
                              a=abuf[shift:], lda=lda, b=bbuf[shift:], ldb=ldb, beta=0.5,
                              c=torch.from_numpy(c).cuda(), ldc=ldc))
            # the oracle reads lda * cols elements: pad the host copies past the last column
            ah = np.concatenate([a.float().numpy(), np.zeros(lda, np.float32)])
            bh = np.concatenate([b.float().numpy(), np.zeros(ldb, np.float32)])
            host.append((ta, tb, m, n, k, 1.0, ah, lda, bh, ldb, 0.5, c, ldc))
    plan = blas.GroupedPlan(sb, probs, dtype="bfloat16")
    plan.run()
    sb.wait()
    _check(probs, host)
    plan.close()
    sb.check_device_error()


@pytest.mark.parametrize("method", ["tcgen05"], indirect=True)
@pytest.mark.parametrize("slices", [2, 9, 64, 65, 152])
def test_grouped_split_k_fold_tree(sb, torch_cuda, method, slices, monkeypatch):
    """Forced slice counts that give fold trees of one, two and three levels
    (fan-in 8), with lone children (9, 65) and ragged output tiles (rows not a
    multiple of 32, N tiles of 2 and 5 columns, whole sub-blocks outside the
    problem): sampled entries against the oracle, and a second run bit for
    bit equal to the first (the tickets reset themselves)."""
    torch = torch_cuda
    from portblas_gb300 import blas
    monkeypatch.setenv("GBBLAS_GROUPED_SPLITK", str(slices))
    g = rng(300 + slices)
    # 3 * slices - 1 or 3 * slices k-blocks of 64: every problem gets exactly `slices` slices
    kb = 3 * slices
    shapes = [(48, 45, (kb - 1) * 64 - 5, False, False), (200, 130, kb * 64, True, False),
              (37, 133, (kb - 1) * 64 + 7, False, True)]
    probs, host = [], []
    for (m, n, k, ta, tb) in shapes:
        lda, ldb, ldc = (k if ta else m) + 1, (n if tb else k) + 2, m + 3
        a = torch.from_numpy(g.uniform(-1, 1, lda * (m if ta else k)).astype(np.float32)).bfloat16()
        b = torch.from_numpy(g.uniform(-1, 1, ldb * (k if tb else n)).astype(np.float32)).bfloat16()
        c = g.uniform(-1, 1, ldc * n).astype(np.float32)
        probs.append(dict(transa="t" if ta else "n", transb="t" if tb else "n", m=m, n=n, k=k, alpha=1.5,
                          a=a.cuda(), lda=lda, b=b.cuda(), ldb=ldb, beta=0.5, c=torch.from_numpy(c).cuda(), ldc=ldc))
        host.append((ta, tb, m, n, k, a.float().numpy(), lda, b.float().numpy(), ldb, c, ldc))
    c0 = [p["c"].clone() for p in probs]
    plan = blas.GroupedPlan(sb, probs, dtype="bfloat16")
    assert plan.info()[1] == slices
    plan.run()
    sb.wait()
    first = [p["c"].clone() for p in probs]
    for p, (ta, tb, m, n, k, a, lda, b, ldb, c, ldc) in zip(probs, host):
        rows = np.concatenate([g.integers(0, m, 40), [m - 1]])
        cols = np.concatenate([g.integers(0, n, 40), [n - 1]])
        ref = oracle.gemm(ta, tb, m, n, k, 1.5, a, lda, b, ldb, 0.5, c, ldc, rows=rows, cols=cols)
        scale = oracle.gemm_absscale(ta, tb, m, n, k, 1.5, a, lda, b, ldb, 0.5, c, ldc, rows=rows, cols=cols)
        out = p["c"].cpu().numpy().reshape(n, ldc).T
        assert (np.abs(out[rows, cols] - ref) / scale).max() <= 1e-5, (m, n, k)
        np.testing.assert_array_equal(out[m:], c.reshape(n, ldc).T[m:])  # padding rows untouched
    for p, c in zip(probs, c0):
        p["c"].copy_(c)
    plan.run()
    sb.wait()
    for p, f in zip(probs, first):
        assert torch.equal(p["c"], f)
    plan.close()
    sb.check_device_error()


@pytest.mark.parametrize("method", ["tcgen05"], indirect=True)
def test_grouped_no_split_for_many_short_problems(sb, torch_cuda, method):
    """Many short problems (no tile dominates the load): no K is split."""
    from portblas_gb300 import blas
    probs, _ = _problems(torch_cuda, rng(73), 200, 16, 400, "float32")
    plan = blas.GroupedPlan(sb, probs, dtype="float32")
    assert plan.info()[1] == 1
    plan.close()


def test_grouped_bf16_transposing_pass_when_mn_tiles_off():
    """With GBBLAS_GROUPED_MN=0 (read once per process, so in a child
    pytest) BF16 operands whose rows are contiguous go through the
    conversion pass's transposing path into K-major tiles: the alignment and
    rows-contiguous cases against the oracle there."""
    import os
    import subprocess
    import sys
    if os.environ.get("GBBLAS_GROUPED_MN") == "0":
        pytest.skip("already the child run")
    env = dict(os.environ, GBBLAS_GROUPED_MN="0")
    here = os.path.dirname(os.path.abspath(__file__))
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider",
                        os.path.join(here, "test_grouped_gpu.py"), "-k",
                        "bf16_operand_alignment or rows_contiguous or bf16_aligned_operands"],
                       env=env, cwd=os.path.dirname(here), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
