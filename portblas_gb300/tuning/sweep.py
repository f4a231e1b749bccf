"""Exhaustive autotuner sweep: times every GEMM configuration of the shape's
element type on seeded random shapes and writes the timing table the
selector is trained on (one row per shape, one column per config; the other
element type's configs are inf).

Shapes: M, N, K = round(2^U(0, 14)) (log-uniform in [1, 16384]), batch =
round(2^U(0, 10)) (log-uniform in [1, 1024]), random transposes, leading
dimensions padded by 1..15 elements half of the time.  Cap: FP32 2*M*N*K*batch
<= 2^35 flop, FP64 <= 2^31 flop (the FP64 pipe is ~40x slower), and every
operand <= 2^27 elements (batch halved first, then the largest dimension) so
one sweep fits a few GPU-minutes; the caps are recorded in the output.  Each
config: one warm-up launch, then CUDA-event timing of `reps` launches (reps
chosen so the timed window is >= ~200 us, at most 10); a config that cannot
take a shape (grid / workspace limits) is recorded as inf.

Run on a GPU:  python -m portblas_gb300.tuning.sweep --shapes 6000 --shapes64 2000 --out FILE.npz
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time

import numpy as np

FLOP_CAP = 2 ** 35
FLOP_CAP64 = 2 ** 31
ELEM_CAP = 2 ** 27
N_CONFIGS, F64_FIRST = 60, 40  # FP32 configs [0, 40), FP64 configs [40, 60)
DTYPE_F32, DTYPE_F64 = 0, 2    # gbblas_dtype_t values


def sample_shapes(count: int, seed: int = 1234, dtype: str = "f32"):
    g = np.random.default_rng(seed)
    cap = FLOP_CAP if dtype == "f32" else FLOP_CAP64
    out = []
    for _ in range(count):
        m, n, k = (int(round(2 ** g.uniform(0, 14))) for _ in range(3))
        b = int(round(2 ** g.uniform(0, 10)))
        ta, tb = int(g.integers(2)), int(g.integers(2))
        while True:
            if 2 * m * n * k * b <= cap and max(m * k, k * n, m * n) * b <= ELEM_CAP:
                break
            if b > 1:
                b = max(1, b // 2)
            else:
                if m >= n and m >= k:
                    m = max(1, m // 2)
                elif n >= k:
                    n = max(1, n // 2)
                else:
                    k = max(1, k // 2)
        pads = [int(g.integers(1, 16)) if g.random() < 0.5 else 0 for _ in range(3)]
        lda = (k if ta else m) + pads[0]
        ldb = (n if tb else k) + pads[1]
        ldc = m + pads[2]
        out.append(dict(m=m, n=n, k=k, batch=b, ta=ta, tb=tb, lda=lda, ldb=ldb, ldc=ldc, dtype=dtype))
    return out


def features(L, s) -> np.ndarray:
    f = (C.c_float * 11)()
    L.gbblas_gemm_features(DTYPE_F64 if s.get("dtype") == "f64" else DTYPE_F32, s["m"], s["n"], s["k"],
                           b"t" if s["ta"] else b"n", b"t" if s["tb"] else b"n", s["lda"], s["ldb"], s["ldc"],
                           s["batch"], C.addressof(f))
    return np.frombuffer(f, dtype=np.float32).copy()


def fit_batch(s, cap_elems: int) -> int:
    """Batch of s after shrinking it so every operand fits `cap_elems`."""
    m, n, k = s["m"], s["n"], s["k"]
    sa = (m * s["lda"]) if s["ta"] else (k * s["lda"])
    sbs = (k * s["ldb"]) if s["tb"] else (n * s["ldb"])
    sc = n * s["ldc"]
    return max(1, min(s["batch"], cap_elems // max(sa, sbs, sc)))


class Runner:
    """Runs config c on shape s with the element type's operand buffers."""

    def __init__(self, L, sb, torch, seed: int, elems: int):
        self.L, self.sb, self.elems = L, sb, elems
        g = torch.Generator(device="cuda").manual_seed(seed)
        self.buf = {}
        for dt, tdt in (("f32", torch.float32), ("f64", torch.float64)):
            A = torch.rand(elems, device="cuda", generator=g, dtype=tdt) - 0.5
            B = torch.rand(elems, device="cuda", generator=g, dtype=tdt) - 0.5
            Cm = torch.zeros(elems + 65536, device="cuda", dtype=tdt)
            self.buf[dt] = (A, B, Cm)

    def configs(self, s):
        return range(0, F64_FIRST) if s.get("dtype", "f32") == "f32" else range(F64_FIRST, N_CONFIGS)

    def run(self, s, c, bt) -> int:
        m, n, k = s["m"], s["n"], s["k"]
        sa = (m * s["lda"]) if s["ta"] else (k * s["lda"])
        sbs = (k * s["ldb"]) if s["tb"] else (n * s["ldb"])
        sc = n * s["ldc"]
        ta, tb = (b"t" if s["ta"] else b"n"), (b"t" if s["tb"] else b"n")
        dt = s.get("dtype", "f32")
        A, B, Cm = self.buf[dt]
        fn = self.L.gbblas_sgemm_strided_batched_config if dt == "f32" else self.L.gbblas_dgemm_strided_batched_config
        return fn(self.sb.handle, c, ta, tb, m, n, k, 1.0, A.data_ptr(), s["lda"], sa, B.data_ptr(), s["ldb"], sbs,
                  0.0, Cm.data_ptr(), s["ldc"], sc, bt)

    def time_all(self, s, e0, e1, min_ms: float = 0.2, max_reps: int = 10) -> np.ndarray:
        """Times every config of s's element type: one warm-up launch, then
        enough launches for a >= min_ms window (at most max_reps)."""
        t = np.full(N_CONFIGS, np.inf, dtype=np.float64)
        bt = fit_batch(s, self.elems - 4096)
        for c in self.configs(s):
            e0.record()
            st = self.run(s, c, bt)
            e1.record()
            if st != 0:
                continue
            e1.synchronize()
            t1 = e0.elapsed_time(e1)
            reps = int(min(max_reps, max(1, math.ceil(min_ms / max(t1, 1e-3)))))
            e0.record()
            for _ in range(reps):
                self.run(s, c, bt)
            e1.record()
            e1.synchronize()
            t[c] = e0.elapsed_time(e1) / reps
        s["batch"] = bt
        return t


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--shapes", type=int, default=6000, help="FP32 shapes")
    ap.add_argument("--shapes64", type=int, default=2000, help="FP64 shapes")
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--out", required=True)
    ap.add_argument("--budget-s", type=float, default=1800.0)
    args = ap.parse_args()
    import torch
    from portblas_gb300 import _lib, blas, build
    build.build()
    L = _lib.load()
    sb = blas.SB_Handle()
    assert L.gbblas_gemm_config_count() == N_CONFIGS
    # FP32 and FP64 shapes interleaved, so a sweep cut short by its budget keeps both
    s32 = sample_shapes(args.shapes, args.seed, "f32")
    s64 = sample_shapes(args.shapes64, args.seed + 1, "f64")
    shapes, i32, i64 = [], 0, 0
    while i32 < len(s32) or i64 < len(s64):
        if i64 < len(s64) and (i32 >= len(s32) or i64 * len(s32) <= i32 * len(s64)):
            shapes.append(s64[i64])
            i64 += 1
        else:
            shapes.append(s32[i32])
            i32 += 1
    R = Runner(L, sb, torch, args.seed, ELEM_CAP + 4096)
    times = np.full((len(shapes), N_CONFIGS), np.inf, dtype=np.float32)
    feats = np.zeros((len(shapes), 11), dtype=np.float32)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_start = time.time()
    done = 0
    for si, s in enumerate(shapes):
        times[si] = R.time_all(s, e0, e1)
        feats[si] = features(L, s)  # after time_all: the batch may have been shrunk
        done = si + 1
        if time.time() - t_start > args.budget_s:
            break
        if done % 250 == 0:
            print(f"{done} shapes, {time.time() - t_start:.0f} s", flush=True)
    sb.check_device_error()
    meta = dict(flop_cap=FLOP_CAP, flop_cap_f64=FLOP_CAP64, elem_cap=ELEM_CAP, seed=args.seed, shapes_done=done,
                seconds=time.time() - t_start, gpu=torch.cuda.get_device_name(),
                sm_count=torch.cuda.get_device_properties(0).multi_processor_count)
    np.savez_compressed(args.out, features=feats[:done], times_ms=times[:done],
                        dtype=np.array([1 if s["dtype"] == "f64" else 0 for s in shapes[:done]], dtype=np.int8),
                        shapes=np.array([[s[k] for k in ("m", "n", "k", "batch", "ta", "tb", "lda", "ldb", "ldc")]
                                         for s in shapes[:done]], dtype=np.int64),
                        meta=json.dumps(meta))
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
