"""Benchmark of the portBLAS hot path on GB300 (one JSON line on rank 0).

Default workload — the memory-bound set, fp32, at its full sizes:
  * _gemv 'n' and 't' on an 8192 x 8192 column-major A (lda 8192, incx = incy
    = 1, alpha 1, beta 0), A ~ U[-1, 1];
  * _asum, _nrm2, _dot, _iamax, _iamin on n = 2^26 vectors ~ N(0, 1), with the
    largest |x| planted at 8 random indices (ties exercise the first-index rule);
  * extension::_reduction Add, inner (column sums) and outer (row sums), over a
    16384 x 16384 matrix.
One step = one pass over all of them.  `value` is the step's algorithmic bytes
(portBLAS's benchmark counters: common/include/common/blas{1,2}_state_counters.hpp)
divided by the device time of the step, inputs resident in HBM; every input is
larger than the 129 MB L2.  `e2e` is the same step through the public API with
host buffers: pinned host->device copies of the inputs and device->host reads of
the results are inside its timed region.  The SGEMM precision/throughput set
(8192^3 NN and TN, entries s*2^u, u ~ U[-10, 10]: plain FP32 SIMT vs split-BF16
on the tensor cores, errors against the FP64 oracle on sampled entries) and
DGEMM 4096^3 are measured in the same run and reported under "sgemm".

Also in the same run: portBLAS's plain SGEMM sample (1024^3 NN, alpha 1.5,
beta 0.5, U[-1, 1)) for AUTO and every FP32 method, under
"config1_sgemm_1024", with OpenBLAS sgemm beside it; the batching set under
"batched"; the learned tile selector under "selector"; and a short "summary"
of the GEMM figures as the line's last key.

--impl reference times the reference's CPU path for the same step on the host
cores: the CBLAS that portBLAS's tests link (numpy's bundled OpenBLAS, all
threads) for GEMV, asum, nrm2 and dot, and FP32 OpenMP restatements of
portBLAS's IndexMax/IndexMin and Reduction kernels (oracle/cpu_baseline.c)
for iamax/iamin (OpenBLAS runs those on one thread) and extension::_reduction
(no CBLAS counterpart).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "SGEMM TFLOP/s split-BF16 vs FP32 @rel err≤1e-6; GEMV/asum GB/s vs HBM peak"
F32 = 4
GEMV_N = 8192
VEC_N = 1 << 26
RED_N = 16384


def algorithmic_bytes() -> dict:
    """Bytes per op, as portBLAS's counters count them."""
    gemv = (GEMV_N * GEMV_N + GEMV_N + GEMV_N) * F32  # A + x + y (beta = 0: y written only)
    return {
        "gemv_n": gemv, "gemv_t": gemv,
        "asum": (VEC_N + 1) * F32, "nrm2": (VEC_N + 1) * F32, "dot": (2 * VEC_N + 1) * F32,
        "iamax": (VEC_N + 1) * F32, "iamin": (VEC_N + 1) * F32,
        "reduction_inner": (RED_N * RED_N + RED_N) * F32, "reduction_outer": (RED_N * RED_N + RED_N) * F32,
    }


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) of
# each kernel of the step, from one ncu --set full capture of
# `bench.py --profile memory --steps 1 --warmup 1` on a GB300, in bytes.
NCU_TRAFFIC = {
    "gemv_n": 0.268490e9 + 3.769088e6, "reduction_outer": 1.073866e9 + 3.405824e6,
    "gemv_t": 0.268530e9 + 4.135424e6, "reduction_inner": 1.073791e9 + 3.998464e6,
    "asum": 268.461312e6 + 3.583232e6, "nrm2": 268.470272e6 + 3.610624e6, "dot": 536.927232e6 + 3.253248e6,
    "iamax": 268.471296e6 + 3.544320e6, "iamin": 268.47e6 + 3.6e6,
}


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "src": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "src": "fallback"}


# ------------------------------------------------------------- clocks --
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------- GPU side --
def make_inputs(torch, dev):
    gen = torch.Generator(device=dev).manual_seed(20240917)
    A = torch.rand(GEMV_N * GEMV_N, device=dev, generator=gen) * 2 - 1
    xg = torch.rand(GEMV_N, device=dev, generator=gen) * 2 - 1
    v = torch.randn(VEC_N, device=dev, generator=gen)
    w = torch.randn(VEC_N, device=dev, generator=gen)
    # plant the largest |x| at 8 distinct random indices with random signs
    pick = np.random.default_rng(20240917)
    idx = torch.from_numpy(pick.choice(VEC_N, size=8, replace=False).astype(np.int64)).to(dev)
    big = 8.0 * v.abs().max()
    signs = torch.from_numpy(pick.choice([-1.0, 1.0], size=8).astype(np.float32)).to(dev)
    v[idx] = big * signs
    R = torch.rand(RED_N * RED_N, device=dev, generator=gen) * 2 - 1
    return dict(A=A, xg=xg, v=v, w=w, R=R, planted=int(idx.min().item()))


def step_ops(blas, sb, inp, outs):
    """The memory-bound set as (name, call) pairs, in step order."""
    return [
        ("gemv_n", lambda: blas._gemv(sb, "n", GEMV_N, GEMV_N, 1.0, inp["A"], GEMV_N, inp["xg"], 1, 0.0,
                                      outs["yn"], 1)),
        ("gemv_t", lambda: blas._gemv(sb, "t", GEMV_N, GEMV_N, 1.0, inp["A"], GEMV_N, inp["xg"], 1, 0.0,
                                      outs["yt"], 1)),
        ("asum", lambda: blas._asum(sb, VEC_N, inp["v"], 1, outs["s"][0:1])),
        ("nrm2", lambda: blas._nrm2(sb, VEC_N, inp["v"], 1, outs["s"][1:2])),
        ("dot", lambda: blas._dot(sb, VEC_N, inp["v"], 1, inp["w"], 1, outs["s"][2:3])),
        ("iamax", lambda: blas._iamax(sb, VEC_N, inp["v"], 1, outs["i"][0:1])),
        ("iamin", lambda: blas._iamin(sb, VEC_N, inp["v"], 1, outs["i"][1:2])),
        ("reduction_inner", lambda: blas.extension._reduction(blas.AddOperator, sb, inp["R"], RED_N, outs["ri"],
                                                              RED_N, RED_N, blas.reduction_dim_t.inner)),
        ("reduction_outer", lambda: blas.extension._reduction(blas.AddOperator, sb, inp["R"], RED_N, outs["ro"],
                                                              RED_N, RED_N, blas.reduction_dim_t.outer)),
    ]


def run_step(blas, sb, inp, outs, events=None):
    """One pass of the memory-bound set; `events` (optional) brackets each op."""
    ops = step_ops(blas, sb, inp, outs)
    for i, (name, fn) in enumerate(ops):
        ev = events.get(name) if events is not None else None
        if ev is not None:
            ev[0].record()
        fn()
        if ev is not None:
            ev[1].record()
    return [n for n, _ in ops]


def bench_memory_set(torch, blas, sb, steps, warmup, dev, record_ops=True):
    inp = make_inputs(torch, dev)
    outs = dict(yn=torch.empty(GEMV_N, device=dev), yt=torch.empty(GEMV_N, device=dev),
                s=torch.zeros(3, device=dev), i=torch.zeros(2, dtype=torch.int32, device=dev),
                ri=torch.empty(RED_N, device=dev), ro=torch.empty(RED_N, device=dev))
    names = list(algorithmic_bytes())
    for _ in range(warmup):
        run_step(blas, sb, inp, outs)
    torch.cuda.synchronize()
    # per-op device times from a short untimed pass (events around each op,
    # steps enqueued back to back; median over the steps after the first)
    per_op = {n: [] for n in names}
    pre = [{n: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for n in names}
           for _ in range(4 if record_ops else 0)]
    for ev in pre:
        run_step(blas, sb, inp, outs, ev)
    torch.cuda.synchronize()
    for ev in pre[1:]:
        for n in names:
            per_op[n].append(ev[n][0].elapsed_time(ev[n][1]))
    dom = max(names, key=lambda n: statistics.median(per_op[n])) if record_ops else None
    # per-op time in a pipeline: PIPE back-to-back calls of one op between two
    # events (the event and launch cost of a lone call, ~4 us, is then spread
    # over the calls).  Consecutive calls alternate between two copies of the
    # inputs, so no call finds its operands in L2; median of three runs
    PIPE = 8
    per_op_pipe = {n: [] for n in names}
    if record_ops:
        inp2 = {k: (v.clone() if hasattr(v, "clone") else v) for k, v in inp.items()}
        pairs = zip(step_ops(blas, sb, inp, outs), step_ops(blas, sb, inp2, outs))
        for (name, fn), (_, fn2) in pairs:
            fn()
            fn2()
            for _ in range(3):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for c in range(PIPE):
                    (fn2 if c & 1 else fn)()
                e1.record()
                torch.cuda.synchronize()
                per_op_pipe[name].append(e0.elapsed_time(e1) / PIPE)
        del inp2, pairs
    # the timed region: K whole steps between two events, enqueued back to
    # back; inside it, two events on the same stream bracket the dominant op
    # of every step (events around all nine ops would slow the step by ~6%)
    dom_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps if record_ops else 0)]
    l0 = blas.launch_count()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        time.sleep(0.3)
        barrier(torch)
        torch.cuda.synchronize()
        start.record()
        for k in range(steps):
            run_step(blas, sb, inp, outs, {dom: dom_ev[k]} if record_ops else None)
        end.record()
        torch.cuda.synchronize()
        barrier(torch)
        time.sleep(0.2)
    launches = blas.launch_count() - l0
    ms = start.elapsed_time(end) / steps
    dom_ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in dom_ev) if record_ops else None
    # correctness of the last step against FP64 (torch, float64 on the GPU)
    iam = outs["i"].cpu().numpy()
    checks = {"iamax_index": int(iam[0]), "iamax_expected_first_planted": inp["planted"]}
    return dict(ms=ms, per_op={n: statistics.median(v) if v else None for n, v in per_op.items()},
                per_op_pipe={n: statistics.median(v) if v else None for n, v in per_op_pipe.items()},
                dom=dom, dom_ms=dom_ms, launches=launches, errors=fp64_errors(torch, inp, outs),
                clocks=clk.summary(), checks=checks, inp=inp, outs=outs)


def barrier(torch) -> None:
    """All ranks meet here when the job is distributed (no-op on one process)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(torch, values, dev):
    """Element-wise maximum of per-rank values (every rank must call it); the
    values themselves on one process."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def fp64_errors(torch, inp, outs):
    """Relative error of each op's result against an FP64 computation of the
    same inputs: vectors as max |got - ref| / max |ref|, scalars as
    |got - ref| / |ref|, indices as an exact match with the first extreme."""
    def vec_err(got, ref):
        return float(((got.double() - ref).abs().max() / ref.abs().max()).item())

    def sca_err(got, ref):
        return float((abs(float(got) - float(ref)) / abs(float(ref))))

    err = {}
    A = inp["A"].view(GEMV_N, GEMV_N).double()  # A[j] = column j
    x = inp["xg"].double()
    err["gemv_n"] = vec_err(outs["yn"], A.T @ x)
    err["gemv_t"] = vec_err(outs["yt"], A @ x)
    del A
    v, w = inp["v"].double(), inp["w"].double()
    s = outs["s"].cpu()
    err["asum"] = sca_err(s[0], v.abs().sum().item())
    err["nrm2"] = sca_err(s[1], v.norm().item())
    err["dot"] = sca_err(s[2], (v * w).sum().item())
    av = inp["v"].abs()
    first = lambda mask: int(torch.nonzero(mask)[0].item())
    iam = outs["i"].cpu()
    err["iamax"] = 0.0 if int(iam[0]) == first(av == av.max()) else 1.0
    err["iamin"] = 0.0 if int(iam[1]) == first(av == av.min()) else 1.0
    del v, w, av
    R = inp["R"].view(RED_N, RED_N).double()  # R[j] = column j
    err["reduction_inner"] = vec_err(outs["ri"], R.sum(1))
    err["reduction_outer"] = vec_err(outs["ro"], R.sum(0))
    del R
    torch.cuda.empty_cache()
    return err


def bench_e2e(torch, blas, sb, steps, warmup, dev):
    """Same step through the public API with host buffers: H2D of every input
    (pinned) and D2H of every result inside the timed region, as a streaming
    caller would run it: the inputs are copied on their own stream into two
    alternating device buffers, each op starts once its own operands have
    landed (GEMV: A and x; BLAS-1: v and w; reductions: R), so step k+1's
    copies overlap step k's kernels; the results go back after every step."""
    g = np.random.default_rng(7)
    host = dict(
        A=torch.from_numpy(g.uniform(-1, 1, GEMV_N * GEMV_N).astype(np.float32)).pin_memory(),
        xg=torch.from_numpy(g.uniform(-1, 1, GEMV_N).astype(np.float32)).pin_memory(),
        v=torch.from_numpy(g.standard_normal(VEC_N).astype(np.float32)).pin_memory(),
        w=torch.from_numpy(g.standard_normal(VEC_N).astype(np.float32)).pin_memory(),
        R=torch.from_numpy(g.uniform(-1, 1, RED_N * RED_N).astype(np.float32)).pin_memory(),
    )
    dev_in = [{k: torch.empty_like(v, device=dev) for k, v in host.items()} for _ in range(2)]
    outs = dict(yn=torch.empty(GEMV_N, device=dev), yt=torch.empty(GEMV_N, device=dev),
                s=torch.zeros(3, device=dev), i=torch.zeros(2, dtype=torch.int32, device=dev),
                ri=torch.empty(RED_N, device=dev), ro=torch.empty(RED_N, device=dev))
    host_out = {k: torch.empty_like(v, device="cpu").pin_memory() for k, v in outs.items()}
    h2d = sum(v.numel() * v.element_size() for v in host.values())
    d2h = sum(v.numel() * v.element_size() for v in outs.values())
    compute = torch.cuda.current_stream()
    copy = torch.cuda.Stream()
    ops = [step_ops(blas, sb, d, outs) for d in dev_in]
    # inputs each op group needs, in step order: 2 GEMVs, 5 BLAS-1, 2 reductions
    groups = [(("A", "xg"), 2), (("v", "w"), 5), (("R",), 2)]
    consumed = [torch.cuda.Event() for _ in range(2)]
    for e in consumed:
        e.record(compute)

    def step(k):
        b = k & 1
        ready = []
        with torch.cuda.stream(copy):
            copy.wait_event(consumed[b])  # the kernels of step k-2 are done with buffer b
            for names, _ in groups:
                for n in names:
                    dev_in[b][n].copy_(host[n], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(copy)
                ready.append(ev)
        i = 0
        for ev, (_, count) in zip(ready, groups):
            compute.wait_event(ev)
            for _, fn in ops[b][i:i + count]:
                fn()
            i += count
        consumed[b].record(compute)
        for n in outs:
            host_out[n].copy_(outs[n], non_blocking=True)

    for k in range(warmup):
        step(k)
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(torch)
    torch.cuda.synchronize()
    start.record(compute)
    copy.wait_event(start)
    for k in range(steps):
        step(warmup + k)
    compute.wait_stream(copy)
    end.record(compute)
    torch.cuda.synchronize()
    barrier(torch)
    # the last step's results, read back through the pipeline, against FP64
    ref_s = float(host["v"].double().abs().sum())
    ok = abs(float(host_out["s"][0]) - ref_s) <= 1e-5 * ref_s
    return dict(ms=start.elapsed_time(end) / steps, h2d=h2d, d2h=d2h, asum_ok=ok)


def bench_sgemm(torch, blas, sb, dev, reps=3, n=8192, with_dgemm=True):
    """n^3 FP32 GEMM (n = 8192 by default): plain SIMT vs split-BF16 (x3 and x6
    products), NN and TN, entries s*2^u (u ~ U[-10, 10]); error against FP64
    dot products (torch, float64 on the GPU) on sampled entries."""
    g = np.random.default_rng(99)

    def pw2(size):
        u = g.uniform(-10, 10, size)
        s = g.choice([-1.0, 1.0], size)
        return (s * np.exp2(u)).astype(np.float32)

    a = pw2(n * n)
    b = pw2(n * n)
    ad, bd = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    cd = torch.zeros(n * n, device=dev)
    rows = g.integers(0, n, 256)
    cols = g.integers(0, n, 256)
    res = {}
    modes = [("fp32_simt", blas.sgemm_mode_t.fp32_simt), ("split_bf16x3", blas.sgemm_mode_t.split_bf16x3),
             ("split_bf16x6", blas.sgemm_mode_t.split_bf16x6)]
    r_t = torch.from_numpy(rows).to(dev)
    c_t = torch.from_numpy(cols).to(dev)
    Bm = bd.view(n, n)  # Bm[j] = column j of B (column-major, ldb = n)
    for ta in (False, True):
        tag = "TN" if ta else "NN"
        # row i of op(A): A is column-major n x n with lda = n
        Am = ad.view(n, n)
        a_rows = (Am[r_t] if ta else Am.T[r_t]).double()  # [256, n]
        b_cols = Bm[c_t].double()                           # [256, n]
        ref = (a_rows * b_cols).sum(1).cpu().numpy()
        scale = (a_rows.abs() * b_cols.abs()).sum(1).cpu().numpy()
        del a_rows, b_cols
        for name, mode in modes:
            sb.set_sgemm_mode(mode)
            try:
                blas._gemm(sb, "t" if ta else "n", "n", n, n, n, 1.0, ad, n, bd, n, 0.0, cd, n)
            except (blas.UnsupportedException, NotImplementedError) as e:
                res[f"{name}_{tag}"] = {"unavailable": str(e)}
                continue
            torch.cuda.synchronize()
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                blas._gemm(sb, "t" if ta else "n", "n", n, n, n, 1.0, ad, n, bd, n, 0.0, cd, n)
                e1.record()
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            got = cd.view(n, n).T.cpu().numpy()[rows, cols].astype(np.float64)
            err = np.abs(got - ref)
            ms = min(ts)
            res[f"{name}_{tag}"] = {
                "tflops": 2.0 * n ** 3 / (ms * 1e-3) / 1e12, "ms": ms,
                "max_rel_err": float(np.max(err / np.maximum(np.abs(ref), 1e-300))),
                "mean_rel_err": float(np.mean(err / np.maximum(np.abs(ref), 1e-300))),
                "max_norm_err": float(np.max(err / scale)), "mean_norm_err": float(np.mean(err / scale)),
                "sampled_entries": len(rows)}
    sb.set_sgemm_mode(blas.sgemm_mode_t.auto)
    if not with_dgemm:
        return res
    # DGEMM 4096^3 on the FP64 pipe
    nd = 4096
    A = torch.rand(nd * nd, device=dev, dtype=torch.float64) * 2 - 1
    B = torch.rand(nd * nd, device=dev, dtype=torch.float64) * 2 - 1
    Cc = torch.zeros(nd * nd, device=dev, dtype=torch.float64)
    blas._gemm(sb, "n", "n", nd, nd, nd, 1.0, A, nd, B, nd, 0.0, Cc, nd)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    blas._gemm(sb, "n", "n", nd, nd, nd, 1.0, A, nd, B, nd, 0.0, Cc, nd)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ref = (A.view(nd, nd).T[:64] @ B.view(nd, nd).T[:, :64])
    derr = float(((Cc.view(nd, nd).T[:64, :64] - ref).abs().max() / ref.abs().max()).item())
    res["dgemm_4096"] = {"tflops": 2.0 * nd ** 3 / (ms * 1e-3) / 1e12, "ms": ms, "max_err_vs_torch_fp64": derr}
    del ad, bd, cd, A, B, Cc
    torch.cuda.empty_cache()
    simt = res.get("fp32_simt_NN", {}).get("tflops")
    for k in ("split_bf16x3_NN", "split_bf16x6_NN"):
        if simt and "tflops" in res.get(k, {}):
            res[k]["speedup_vs_fp32_simt"] = res[k]["tflops"] / simt
    return res


FP32_SIMT_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12  # nominal: SMs x FP32 lanes x FMA x max SM clock


def l2_flush(torch, buf):
    """Evicts the 129 MB L2 between timed calls by writing a larger buffer."""
    buf.add_(1.0)


def bench_config1(torch, blas, sb, dev, reps=30):
    """portBLAS's plain SGEMM sample (samples/gemm.cpp:22-23): C <- 1.5 A B +
    0.5 C, NN, M = N = K = 1024, ld 1024, entries U[-1, 1) from a fixed seed,
    for AUTO and every FP32 method; each timed call between CUDA events after
    an L2 flush (median); error of the whole C against FP64 (torch float64 on
    the GPU) as max |C - C64| / (1.5 |A||B| + 0.5 |C_in|).  CPU baseline:
    OpenBLAS sgemm on all host threads."""
    import ctypes as C
    from portblas_gb300 import _lib
    L = _lib.load()
    n = 1024
    g = np.random.default_rng(1024)
    a = g.uniform(-1, 1, n * n).astype(np.float32)
    b = g.uniform(-1, 1, n * n).astype(np.float32)
    c0 = g.uniform(-1, 1, n * n).astype(np.float32)
    ad, bd, c0d = (torch.from_numpy(x).to(dev) for x in (a, b, c0))
    A64, B64, C64 = (x.double().view(n, n).T for x in (ad, bd, c0d))
    ref = 1.5 * (A64 @ B64) + 0.5 * C64
    scale = 1.5 * (A64.abs() @ B64.abs()) + 0.5 * C64.abs()
    del A64, B64, C64
    flush = torch.empty(64 << 20, device=dev)  # 256 MB
    flop = 2.0 * n ** 3
    pk = peaks()
    pick = C.c_int(-1)
    L.gbblas_sgemm_selector_pick(n, n, n, b"n", b"n", n, n, n, 1, C.byref(pick))
    out = {"workload": "sgemm NN 1024^3 alpha 1.5 beta 0.5 ld 1024, U[-1,1)", "auto_config": pick.value,
           "l2": "flushed before every timed call"}
    cd = torch.empty_like(c0d)
    for name in ("auto", "fp32_simt", "split_bf16x3", "split_bf16x6"):
        sb.set_sgemm_mode(getattr(blas.sgemm_mode_t, name))
        cd.copy_(c0d)
        blas._gemm(sb, "n", "n", n, n, n, 1.5, ad, n, bd, n, 0.5, cd, n)
        err = ((cd.double().view(n, n).T - ref).abs() / scale).max().item()
        ts = []
        for i in range(reps + 3):
            l2_flush(torch, flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            blas._gemm(sb, "n", "n", n, n, n, 1.5, ad, n, bd, n, 0.5, cd, n)
            e1.record()
            e1.synchronize()
            if i >= 3:
                ts.append(e0.elapsed_time(e1))
        ms = statistics.median(ts)
        tf = flop / (ms * 1e-3) / 1e12
        r = {"ms": ms, "tflops": tf, "max_norm_err_vs_fp64": err}
        if name == "fp32_simt":
            r["roofline"] = {"bound": "fp32 pipe", "peak": FP32_SIMT_PEAK_TFLOPS, "peak_src": "nominal",
                             "frac": tf / FP32_SIMT_PEAK_TFLOPS}
        elif name.startswith("split"):
            prods = 3 if name.endswith("x3") else 6
            r["roofline"] = {"bound": "tensor", "mma_tflops": prods * tf, "peak": pk["bf16_tflops"],
                             "peak_src": pk["src"] + " bf16 burst", "frac": prods * tf / pk["bf16_tflops"]}
        out[name] = r
    sb.set_sgemm_mode(blas.sgemm_mode_t.auto)
    del flush
    torch.cuda.empty_cache()
    return out


def cpu_config1(budget_s: float = 10.0) -> dict:
    """OpenBLAS sgemm 1024^3 NN (alpha 1.5, beta 0.5) on all host threads, median."""
    import oracle
    cb = oracle.CBlas()
    cb.set_threads(os.cpu_count() or 1)
    n = 1024
    g = np.random.default_rng(1024)
    a = g.uniform(-1, 1, n * n).astype(np.float32)
    b = g.uniform(-1, 1, n * n).astype(np.float32)
    c = g.uniform(-1, 1, n * n).astype(np.float32)
    for _ in range(3):
        cb.sgemm(False, False, n, n, n, 1.5, a, n, b, n, 0.5, c, n)
    ts, t_start = [], time.perf_counter()
    while len(ts) < 10 and time.perf_counter() - t_start < budget_s:
        t0 = time.perf_counter()
        cb.sgemm(False, False, n, n, n, 1.5, a, n, b, n, 0.5, c, n)
        ts.append(time.perf_counter() - t0)
    ms = statistics.median(ts) * 1e3
    return {"tflops": 2.0 * n ** 3 / (ms * 1e-3) / 1e12, "ms": ms, "cores": os.cpu_count() or 1,
            "kind": "port", "sample": f"OpenBLAS sgemm 1024^3 NN, {len(ts)} calls, median"}


def bench_batched(torch, blas, sb, dev, reps=10):
    """Batching workload: a grouped batch of 2048 problems with M, N, K each
    log-uniform in [16, 512] (seeded), random transposes, FP32 and BF16 inputs
    (FP32 accumulate), as one persistent launch replayed from a CUDA graph;
    and a strided batch of 4096 x 64^3 FP32."""
    g = np.random.default_rng(4)
    count = 2048
    dims = np.round(np.exp(g.uniform(np.log(16), np.log(512), (count, 3)))).astype(int)
    trans = g.integers(0, 2, (count, 2))
    flops = float(2 * np.prod(dims, axis=1).sum())
    out = {"grouped": {"problems": count, "flop_per_call": flops}}
    for dt in ("float32", "bfloat16"):
        tdt = torch.float32 if dt == "float32" else torch.bfloat16
        probs, bytes_in = [], 0
        for (m, n, k), (ta, tb) in zip(dims, trans):
            a = torch.rand(int(m * k), device=dev, dtype=torch.float32).to(tdt)
            b = torch.rand(int(k * n), device=dev, dtype=torch.float32).to(tdt)
            c = torch.empty(int(m * n), device=dev)
            bytes_in += a.numel() * a.element_size() + b.numel() * b.element_size() + c.numel() * 4
            probs.append(dict(transa="t" if ta else "n", transb="t" if tb else "n", m=int(m), n=int(n), k=int(k),
                              alpha=1.0, a=a, lda=int(k if ta else m), b=b, ldb=int(n if tb else k), beta=0.0, c=c,
                              ldc=int(m)))
        plan = blas.GroupedPlan(sb, probs, dtype=dt)
        for _ in range(3):
            plan.run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            plan.run()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out["grouped"][dt] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12,
                              "gbs": bytes_in / (ms * 1e-3) / 1e9, "bytes_per_call": bytes_in,
                              "max_norm_err_vs_fp64": grouped_error(torch, probs[::128])}
        plan.close()
        del probs
    out["strided_4096x64"] = bench_strided(torch, blas, sb, dev, reps)
    out["grouped_splitk"] = bench_grouped_splitk(torch, blas, sb, dev, reps)
    return out


def bench_strided(torch, blas, sb, dev, reps=10):
    """Strided batch of 4096 FP32 problems of 64^3 (A, B, C 64 MiB each,
    inputs U[0, 1)); error of three problems against FP64, |A||B|-normalised."""
    nb, n = 4096, 64
    A = torch.rand(nb * n * n, device=dev)
    B = torch.rand(nb * n * n, device=dev)
    Cc = torch.empty(nb * n * n, device=dev)
    f = 2.0 * nb * n ** 3
    byt = 3 * nb * n * n * 4
    sb.set_sgemm_mode(blas.sgemm_mode_t.auto)
    for _ in range(3):
        blas._gemm_strided_batched(sb, "n", "n", n, n, n, 1.0, A, n, n * n, B, n, n * n, 0.0, Cc, n, n * n, nb)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        blas._gemm_strided_batched(sb, "n", "n", n, n, n, 1.0, A, n, n * n, B, n, n * n, 0.0, Cc, n, n * n, nb)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    errs = []
    for i in (0, nb // 2, nb - 1):  # |A||B|-normalised error of three problems against FP64
        Ai = A[i * n * n:(i + 1) * n * n].view(n, n).T.double()
        Bi = B[i * n * n:(i + 1) * n * n].view(n, n).T.double()
        ref = Ai @ Bi
        scale = Ai.abs() @ Bi.abs()
        errs.append(float(((Cc[i * n * n:(i + 1) * n * n].view(n, n).T.double() - ref).abs() / scale).max().item()))
    return {"ms": ms, "tflops": f / (ms * 1e-3) / 1e12, "gbs": byt / (ms * 1e-3) / 1e9, "bytes_per_call": byt,
            "max_norm_err_vs_fp64": max(errs)}


SPLITK_CASES = {
    "tall_skinny_48x48x2^18": [(48, 48, 1 << 18)],
    "4x_128x128x65536": [(128, 128, 65536)] * 4,
    "16x_256x256x32768": [(256, 256, 32768)] * 16,
    "2_long_64_short": [(200, 130, 40000), (64, 64, 100000)] + [(100, 100, 200)] * 64,
}


def bench_grouped_splitk(torch, blas, sb, dev, reps=10):
    """Long-K grouped batches (few output tiles, K up to 2^18): the plan's
    split-K schedule against the same plan with split-K off
    (GBBLAS_GROUPED_SPLITK=0), FP32 and BF16 inputs, uniform [0, 1) data;
    error of the first problem against FP64."""
    out = {}
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    for dt in ("bfloat16", "float32"):
        tdt = torch.float32 if dt == "float32" else torch.bfloat16
        for name, shapes in SPLITK_CASES.items():
            probs = []
            for (m, n, k) in shapes:
                a = torch.rand(m * k, device=dev, generator=g).to(tdt)
                b = torch.rand(k * n, device=dev, generator=g).to(tdt)
                probs.append(dict(transa="n", transb="n", m=m, n=n, k=k, alpha=1.0, a=a, lda=m, b=b, ldb=k,
                                  beta=0.0, c=torch.empty(m * n, device=dev), ldc=m))
            flop = sum(2.0 * m * n * k for (m, n, k) in shapes)
            res = {}
            for mode in ("split", "no_split"):
                old = os.environ.get("GBBLAS_GROUPED_SPLITK")
                os.environ["GBBLAS_GROUPED_SPLITK"] = "1" if mode == "split" else "0"
                try:
                    plan = blas.GroupedPlan(sb, probs, dtype=dt)
                finally:
                    if old is None:
                        del os.environ["GBBLAS_GROUPED_SPLITK"]
                    else:
                        os.environ["GBBLAS_GROUPED_SPLITK"] = old
                tiles, splits = plan.info()
                for _ in range(3):
                    plan.run()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    plan.run()
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / reps
                m, n, k = shapes[0]
                p = probs[0]
                ref = p["a"].double().view(k, m).T @ p["b"].double().view(n, k).T
                err = float(((p["c"].double().view(n, m).T - ref).abs() / ref.abs()).max().item())
                res[mode] = {"ms": ms, "tflops": flop / (ms * 1e-3) / 1e12, "tiles": tiles, "max_splits": splits,
                             "max_rel_err_vs_fp64": err}
                plan.close()
            out[f"{dt}:{name}"] = res
    return out


def grouped_error(torch, probs):
    """Largest |A||B|-normalised error of the given grouped problems (column-
    major, alpha = 1, beta = 0) against FP64 products on the GPU."""
    worst = 0.0
    for p in probs:
        m, n, k = p["m"], p["n"], p["k"]
        # column-major storage: op(A) is m x k, op(B) is k x n
        if p["transa"] == "n":
            a = p["a"].double().view(k, p["lda"])[:, :m].T
        else:
            a = p["a"].double().view(m, p["lda"])[:, :k]
        if p["transb"] == "n":
            b = p["b"].double().view(n, p["ldb"])[:, :k].T
        else:
            b = p["b"].double().view(k, p["ldb"])[:, :n]
        ref = a @ b
        scale = a.abs() @ b.abs()
        got = p["c"].double().view(n, p["ldc"]).T[:m]
        worst = max(worst, float(((got - ref).abs() / scale.clamp_min(1e-300)).max().item()))
    return worst


def bench_selector(torch, blas, sb, dev, n32=200, n64=50):
    """Learned tile selector, measured live: on fresh seeded shapes (seeds
    not in the training sweep; FP32 and FP64, the sweep's distributions and
    caps) every config of the shape's element type is timed exhaustively and
    the regret t(pick)/t(best) - 1 of the learned selector and of the size
    heuristic is averaged per element type.  The held-out figures of the
    training run (tuning/gemm_selector_report.json) are reported beside."""
    import ctypes as C
    from portblas_gb300 import _lib
    from portblas_gb300.tuning import sweep
    L = _lib.load()
    rep_path = os.path.join(ROOT, "portblas_gb300", "tuning", "gemm_selector_report.json")
    report = json.load(open(rep_path)) if os.path.exists(rep_path) else None
    R = sweep.Runner(L, sb, torch, 987654, sweep.ELEM_CAP + 4096)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    for dt, count, seed in (("f32", n32, 987654), ("f64", n64, 987655)):
        r_mlp, r_heur = [], []
        for s in sweep.sample_shapes(count, seed=seed, dtype=dt):
            t = R.time_all(s, e0, e1, min_ms=0.1, max_reps=5)
            if not np.isfinite(t).any():
                continue
            code = sweep.DTYPE_F64 if dt == "f64" else sweep.DTYPE_F32
            pick = C.c_int()
            L.gbblas_gemm_selector_pick(code, s["m"], s["n"], s["k"], b"t" if s["ta"] else b"n",
                                        b"t" if s["tb"] else b"n", s["lda"], s["ldb"], s["ldc"], s["batch"],
                                        C.byref(pick))
            h = L.gbblas_gemm_heuristic_config(code, s["m"], s["n"], s["k"], s["batch"])
            r_mlp.append(t[pick.value] / t.min() - 1)
            r_heur.append(t[h] / t.min() - 1)
        out[dt] = {"live_shapes": len(r_mlp), "regret_mean": {"mlp": float(np.mean(r_mlp)),
                                                              "heuristic": float(np.mean(r_heur))},
                   "regret_median_mlp": float(np.median(r_mlp))}
    res = {"live": out}
    if report:
        res["heldout_training_run"] = {
            "shapes": report.get("heldout_shapes"), "regret_mean": report.get("regret_mean"),
            "per_dtype": {k: v and v["regret_mean"] for k, v in report.get("per_dtype", {}).items()}}
    return res


def summarize(c1, sg, bat, sel, pk) -> dict | None:
    """The GEMM and batching headline figures in a few hundred bytes."""
    if sg is None:
        return None
    r3 = lambda x: None if x is None else float(f"{x:.3g}")
    out = {}
    nn = {k: sg.get(f"{k}_NN", {}) for k in ("fp32_simt", "split_bf16x3", "split_bf16x6")}
    tn = {k: sg.get(f"{k}_TN", {}) for k in ("fp32_simt", "split_bf16x3", "split_bf16x6")}
    x3 = nn["split_bf16x3"]
    out["sgemm8192_tflops"] = {k: r3(v.get("tflops")) for k, v in nn.items()}
    out["sgemm8192_max_norm_err"] = {k: r3(max(v.get("max_norm_err", 0), tn[k].get("max_norm_err", 0)))
                                     for k, v in nn.items()}
    if x3.get("tflops") and nn["fp32_simt"].get("tflops"):
        out["x3_speedup_vs_simt"] = r3(x3["tflops"] / nn["fp32_simt"]["tflops"])
        # the dense x3 kernel issues three BF16 products per FP32 flop
        out["x3_roofline"] = {"bound": "tensor", "achieved": r3(3 * x3["tflops"]), "peak": pk["bf16_tflops"],
                              "unit": "TFLOP/s", "frac": r3(3 * x3["tflops"] / pk["bf16_tflops"]),
                              "peak_src": pk["src"] + " bf16 burst"}
    out["err_measure"] = "max |C-C64| / (|alpha||A||B| + |beta||C|)"
    if "dgemm_4096" in sg:
        out["dgemm4096_tflops"] = r3(sg["dgemm_4096"]["tflops"])
    if c1:
        out["config1"] = {k: {"tflops": r3(c1[k]["tflops"]), "err": r3(c1[k]["max_norm_err_vs_fp64"])}
                          for k in ("auto", "fp32_simt", "split_bf16x3", "split_bf16x6")}
        if c1.get("cpu_baseline"):
            out["config1"]["cpu_openblas_tflops"] = r3(c1["cpu_baseline"]["tflops"])
    if bat:
        gr = bat["grouped"]
        out["grouped2048"] = {dt: {"ms": r3(gr[dt]["ms"]), "tflops": r3(gr[dt]["tflops"]),
                                   "err": r3(gr[dt]["max_norm_err_vs_fp64"])} for dt in ("float32", "bfloat16")}
        st = bat["strided_4096x64"]
        out["strided4096x64"] = {"ms": r3(st["ms"]), "gbs": r3(st["gbs"]), "hbm_frac": r3(st["gbs"] / pk["hbm_gbs"]),
                                 "err": r3(st["max_norm_err_vs_fp64"])}
    if sel:
        out["selector_regret_live"] = {dt: {"mlp": r3(v["regret_mean"]["mlp"]), "heuristic": r3(v["regret_mean"]["heuristic"]),
                                            "shapes": v["live_shapes"]} for dt, v in sel["live"].items()}
    return out


# ----------------------------------------------------------- CPU side --
def cpu_reference_step(cb, oracle_mod, data, outs):
    """The memory-bound step on the host cores: OpenBLAS CBLAS (all threads)
    for GEMV, asum, nrm2 and dot; the FP32 OpenMP restatements of portBLAS's
    IndexMax/IndexMin and Reduction kernels (oracle/cpu_baseline.c) for
    iamax/iamin (OpenBLAS runs those on one thread) and the reductions (no
    CBLAS counterpart)."""
    cb.sgemv("n", GEMV_N, GEMV_N, 1.0, data["A"], GEMV_N, data["xg"], 1, 0.0, outs["yn"], 1)
    cb.sgemv("t", GEMV_N, GEMV_N, 1.0, data["A"], GEMV_N, data["xg"], 1, 0.0, outs["yt"], 1)
    cb.sasum(VEC_N, data["v"], 1)
    cb.snrm2(VEC_N, data["v"], 1)
    cb.sdot(VEC_N, data["v"], 1, data["w"], 1)
    oracle_mod.cpu_iamax(data["v"], is_min=False)
    oracle_mod.cpu_iamax(data["v"], is_min=True)
    oracle_mod.cpu_reduction_add("inner", data["R"], RED_N, RED_N, RED_N, out=outs["ri"])
    oracle_mod.cpu_reduction_add("outer", data["R"], RED_N, RED_N, RED_N, out=outs["ro"])


CPU_SAMPLE = ("OpenBLAS CBLAS on all host threads (sgemv N/T, sasum, snrm2, sdot) + FP32 OpenMP restatements "
              "of portBLAS IndexMax/IndexMin (iamax, iamin) and Reduction (inner + outer, FP32 accumulate, "
              "FP32 input)")


def cpu_reference_data():
    g = np.random.default_rng(3)
    return dict(A=g.uniform(-1, 1, GEMV_N * GEMV_N).astype(np.float32),
                xg=g.uniform(-1, 1, GEMV_N).astype(np.float32),
                v=g.standard_normal(VEC_N).astype(np.float32), w=g.standard_normal(VEC_N).astype(np.float32),
                R=g.uniform(-1, 1, RED_N * RED_N).astype(np.float32))


def bench_cpu(steps: int, warmup: int, budget_s: float = 20.0) -> dict:
    import oracle
    cores = os.cpu_count() or 1
    cb = oracle.CBlas()
    cb.set_threads(cores)
    data = cpu_reference_data()
    outs = dict(yn=np.empty(GEMV_N, np.float32), yt=np.empty(GEMV_N, np.float32),
                ri=np.empty(RED_N, np.float32), ro=np.empty(RED_N, np.float32))
    for _ in range(max(1, warmup)):
        cpu_reference_step(cb, oracle, data, outs)
    ts = []
    t_start = time.perf_counter()
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        cpu_reference_step(cb, oracle, data, outs)
        ts.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > budget_s:
            break
    ms = statistics.median(ts) * 1e3
    total = sum(algorithmic_bytes().values())
    return dict(value=total / (ms * 1e-3) / 1e9, ms=ms, cores=cores, threads_oracle=oracle.num_threads(),
                steps=len(ts))


# --------------------------------------------------------------- main --
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbblas", choices=["gbblas", "reference"])
    ap.add_argument("--no-sgemm", action="store_true", help="skip the SGEMM/DGEMM set")
    ap.add_argument("--profile", choices=["memory", "sgemm", "batched", "strided"], default=None,
                    help="short run of one workload only (no e2e, CPU baseline or JSON line), for ncu captures")
    ap.add_argument("--sgemm-n", type=int, default=8192)
    args = ap.parse_args()
    warmup = max(3, args.warmup)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    total_bytes = sum(algorithmic_bytes().values())
    config = {"workload": "memory-bound set fp32: gemv N+T 8192^2, asum/nrm2/dot/iamax/iamin n=2^26, "
                          "reduction Add inner+outer 16384^2",
              "gemv": [GEMV_N, GEMV_N], "vector_n": VEC_N, "reduction": [RED_N, RED_N],
              "bytes_per_step": total_bytes, "l2": "every input larger than L2 (no flush needed)",
              "parallelism": f"replicas{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        r = bench_cpu(args.steps, args.warmup)
        line = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": "GB/s", "n_gpus": args.gpus,
                "steps": r["steps"], "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": config,
                "cpu_baseline": {"value": r["value"], "unit": "GB/s", "cores": r["cores"], "kind": "port",
                                 "sample": f"{r['steps']} full memory-bound steps on the host, median: " + CPU_SAMPLE},
                "e2e": {"value": r["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    dev = torch.device("cuda", torch.cuda.current_device())
    import __graft_entry__
    __graft_entry__.build()
    from portblas_gb300 import blas
    sb = blas.SB_Handle()
    if args.profile == "memory":
        r = bench_memory_set(torch, blas, sb, args.steps, args.warmup, dev, record_ops=False)
        print(json.dumps({"profile": "memory", "ms_per_step": r["ms"]}))
        return
    if args.profile == "batched":
        print(json.dumps({"profile": "batched", "res": bench_batched(torch, blas, sb, dev, reps=2)}))
        return
    if args.profile == "strided":
        print(json.dumps({"profile": "strided", "res": bench_strided(torch, blas, sb, dev, reps=args.steps)}))
        return
    if args.profile == "sgemm":
        r = bench_sgemm(torch, blas, sb, dev, reps=1, n=args.sgemm_n, with_dgemm=False)
        print(json.dumps({"profile": "sgemm", "n": args.sgemm_n, "res": r}))
        return
    mem = bench_memory_set(torch, blas, sb, args.steps, warmup, dev)
    e2e = bench_e2e(torch, blas, sb, max(3, args.steps // 4), 3, dev)
    ms = mem["ms"]
    ms, e2e_ms = max_over_ranks(torch, [ms, e2e["ms"]], dev)
    value = world * total_bytes / (ms * 1e-3) / 1e9
    pk = peaks()
    ab = algorithmic_bytes()
    dom = mem["dom"]
    achieved = ab[dom] / (mem["dom_ms"] * 1e-3) / 1e9  # its mean launch duration inside the timed region
    sg = bat = sel = c1 = None
    if not args.no_sgemm:
        c1 = bench_config1(torch, blas, sb, dev)
        sg = bench_sgemm(torch, blas, sb, dev)
        bat = bench_batched(torch, blas, sb, dev)
        sel = bench_selector(torch, blas, sb, dev)
    if rank != 0:
        return
    cpu = bench_cpu(2, 1, budget_s=15.0)
    if c1 is not None:
        c1["cpu_baseline"] = cpu_config1()
    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)", "config": config,
        "hbm_frac_of_" + pk["src"]: value / world / pk["hbm_gbs"],
        # per op: "ms" / "gbs" / "frac" from 8 back-to-back calls between two
        # events; "*_single_call" from one call between two events
        "per_op": {n: {"ms": tp, "gbs": ab[n] / (tp * 1e-3) / 1e9, "frac": ab[n] / (tp * 1e-3) / 1e9 / pk["hbm_gbs"],
                       "ms_single_call": t, "frac_single_call": ab[n] / (t * 1e-3) / 1e9 / pk["hbm_gbs"],
                       "rel_err_vs_fp64": mem["errors"].get(n)}
                   for n, t in mem["per_op"].items() for tp in [mem["per_op_pipe"][n]]},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "peak_src": pk["src"],
                     "traffic": NCU_TRAFFIC.get(dom), "traffic_unit": "bytes per launch (ncu)",
                     "algorithmic_bytes": ab[dom]},
        "e2e": {"value": world * total_bytes / (e2e_ms * 1e-3) / 1e9, "unit": "GB/s",
                "h2d_bytes_per_step": e2e["h2d"], "d2h_bytes_per_step": e2e["d2h"],
                "pipelined": "inputs copied on a second stream into two alternating buffers; "
                             "step k+1's copies overlap step k's kernels",
                "last_asum_matches_fp64": e2e["asum_ok"]},
        "gpu_launches": mem["launches"], "clocks": mem["clocks"], "checks": mem["checks"],
        "cpu_baseline": {"value": cpu["value"], "unit": "GB/s", "cores": cpu["cores"], "kind": "port",
                         "sample": f"{cpu['steps']} full memory-bound steps on the host, median: " + CPU_SAMPLE},
        "config1_sgemm_1024": c1,
        "sgemm": sg,
        "batched": bat,
        "selector": sel,
    }
    line["summary"] = summarize(c1, sg, bat, sel, pk)  # last key: short, so that a cut tail still holds it
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
