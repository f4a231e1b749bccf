"""Exhaustive autotuner sweep: times every FP32 GEMM configuration on seeded
random shapes and writes the timing table the selector is trained on.

Shapes: M, N, K = round(2^U(0, 14)) (log-uniform in [1, 16384]), batch =
round(2^U(0, 10)) (log-uniform in [1, 1024]), random transposes, leading
dimensions padded by 1..15 elements half of the time.  Cap: 2*M*N*K*batch
<= 2^35 flop and every operand <= 2^27 elements (batch halved first, then the
largest dimension) so one sweep fits a few GPU-minutes; the cap is recorded
in the output.  Each config: one warm-up launch, then CUDA-event timing of
`reps` launches (reps chosen so the timed window is >= ~200 us, at most 10);
a config that cannot take a shape (grid / workspace limits) is recorded as
inf.

Run on a GPU:  python -m portblas_gb300.tuning.sweep --shapes 6000 --out FILE.npz
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time

import numpy as np

FLOP_CAP = 2 ** 35
ELEM_CAP = 2 ** 27


def sample_shapes(count: int, seed: int = 1234):
    g = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        m, n, k = (int(round(2 ** g.uniform(0, 14))) for _ in range(3))
        b = int(round(2 ** g.uniform(0, 10)))
        ta, tb = int(g.integers(2)), int(g.integers(2))
        while True:
            if 2 * m * n * k * b <= FLOP_CAP and max(m * k, k * n, m * n) * b <= ELEM_CAP:
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
        out.append(dict(m=m, n=n, k=k, batch=b, ta=ta, tb=tb, lda=lda, ldb=ldb, ldc=ldc))
    return out


def features(L, s) -> np.ndarray:
    f = (C.c_float * 11)()
    L.gbblas_sgemm_features(s["m"], s["n"], s["k"], b"t" if s["ta"] else b"n", b"t" if s["tb"] else b"n",
                            s["lda"], s["ldb"], s["ldc"], s["batch"], C.addressof(f))
    return np.frombuffer(f, dtype=np.float32).copy()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--shapes", type=int, default=6000)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--out", required=True)
    ap.add_argument("--budget-s", type=float, default=1800.0)
    args = ap.parse_args()
    import torch
    from portblas_gb300 import _lib, blas, build
    build.build()
    L = _lib.load()
    sb = blas.SB_Handle()
    ncfg = L.gbblas_sgemm_config_count()
    shapes = sample_shapes(args.shapes, args.seed)
    g = torch.Generator(device="cuda").manual_seed(args.seed)
    A = torch.rand(ELEM_CAP + 4096, device="cuda", generator=g) - 0.5
    B = torch.rand(ELEM_CAP + 4096, device="cuda", generator=g) - 0.5
    Cm = torch.zeros(ELEM_CAP + 4096 * 16, device="cuda")
    times = np.full((len(shapes), ncfg), np.inf, dtype=np.float32)
    feats = np.zeros((len(shapes), 11), dtype=np.float32)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_start = time.time()
    done = 0
    for si, s in enumerate(shapes):
        feats[si] = features(L, s)
        m, n, k, bt = s["m"], s["n"], s["k"], s["batch"]
        sa = (m * s["lda"]) if s["ta"] else (k * s["lda"])
        sbs = (k * s["ldb"]) if s["tb"] else (n * s["ldb"])
        sc = n * s["ldc"]
        if max(sa, sbs, sc) * bt > ELEM_CAP + 4096:
            # ld padding can push a capped shape just over: shrink the batch
            bt = max(1, (ELEM_CAP + 4096) // max(sa, sbs, sc))
            s["batch"] = bt
            feats[si] = features(L, s)
        ta, tb = (b"t" if s["ta"] else b"n"), (b"t" if s["tb"] else b"n")

        def run(c):
            return L.gbblas_sgemm_strided_batched_config(sb.handle, c, ta, tb, m, n, k, 1.0, A.data_ptr(),
                                                         s["lda"], sa, B.data_ptr(), s["ldb"], sbs, 0.0,
                                                         Cm.data_ptr(), s["ldc"], sc, bt)

        for c in range(ncfg):
            e0.record()
            st = run(c)
            e1.record()
            if st != 0:
                continue
            e1.synchronize()
            t1 = e0.elapsed_time(e1)
            reps = int(min(10, max(1, math.ceil(0.2 / max(t1, 1e-3)))))
            e0.record()
            for _ in range(reps):
                run(c)
            e1.record()
            e1.synchronize()
            times[si, c] = e0.elapsed_time(e1) / reps
        done = si + 1
        if time.time() - t_start > args.budget_s:
            break
        if done % 250 == 0:
            print(f"{done} shapes, {time.time() - t_start:.0f} s", flush=True)
    sb.check_device_error()
    meta = dict(flop_cap=FLOP_CAP, elem_cap=ELEM_CAP, seed=args.seed, shapes_done=done,
                seconds=time.time() - t_start, gpu=torch.cuda.get_device_name(),
                sm_count=torch.cuda.get_device_properties(0).multi_processor_count)
    np.savez_compressed(args.out, features=feats[:done], times_ms=times[:done],
                        shapes=np.array([[s[k] for k in ("m", "n", "k", "batch", "ta", "tb", "lda", "ldb", "ldc")]
                                         for s in shapes[:done]], dtype=np.int64),
                        meta=json.dumps(meta))
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
