"""Trains the FP32 GEMM tile selector on a sweep's timing table with the
library's own CUDA kernels (gbblas_mlp_loss_grad / gbblas_mlp_adam), then
measures its regret against exhaustive autotuning on held-out shapes.

Target: for each shape and config, log2(t_config / t_best), clipped at 8
(configs that cannot run are masked out).  Selection = argmin of the
predicted targets.  Regret of a selector on a shape = t(pick)/t(best) - 1.

Run on a GPU:
  python -m portblas_gb300.tuning.train --sweep FILE.npz --out-dir DIR
writes DIR/sgemm_selector.bin (the weights the library loads) and
DIR/sgemm_selector_report.json.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import struct
import time

import numpy as np

IN, HID, OUT = 11, 64, 40
CLIP = 8.0


def init_params(seed: int) -> np.ndarray:
    g = np.random.default_rng(seed)
    dims = [IN, HID, HID, HID, OUT]
    parts = []
    for l in range(4):
        fan_in = dims[l]
        parts.append((g.standard_normal((dims[l + 1], dims[l])) * np.sqrt(2.0 / fan_in)).astype(np.float32).ravel())
        parts.append(np.zeros(dims[l + 1], np.float32))
    return np.concatenate(parts)


def targets(times: np.ndarray):
    best = np.min(times, axis=1, keepdims=True)
    ok = np.isfinite(times)
    rel = np.where(ok, np.log2(np.maximum(times, 1e-9) / best), CLIP)
    return np.minimum(rel, CLIP).astype(np.float32), ok.astype(np.float32)


def regret(times: np.ndarray, picks: np.ndarray) -> np.ndarray:
    best = np.min(times, axis=1)
    t = times[np.arange(len(picks)), picks]
    return t / best - 1.0


def write_bin(path: str, params: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(b"GBMLP\0\0\0")
        f.write(struct.pack("<3i", IN, HID, OUT))
        f.write(params.astype("<f4").tobytes())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sweep", required=True)
    ap.add_argument("--out-dir", required=True)
    ap.add_argument("--train", type=int, default=5000)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=7)
    args = ap.parse_args()
    import torch
    from portblas_gb300 import _lib, blas, build
    build.build()
    L = _lib.load()
    sb = blas.SB_Handle()
    d = np.load(args.sweep)
    X = d["features"].astype(np.float32)
    T = d["times_ms"].astype(np.float64)
    keep = np.isfinite(T).any(axis=1)
    X, T, shapes = X[keep], T[keep], d["shapes"][keep]
    Y, Mk = targets(T)
    ntr = min(args.train, len(X) - 1)
    Xtr, Ytr, Mtr = X[:ntr], Y[:ntr], Mk[:ntr]
    Xte, Tte = X[ntr:], T[ntr:]

    cnt = C.c_int64()
    L.gbblas_mlp_param_count(IN, HID, OUT, C.byref(cnt))
    p0 = init_params(args.seed)
    assert p0.size == cnt.value
    dev = "cuda"
    P = torch.from_numpy(p0).to(dev)
    G = torch.zeros_like(P)
    Mo, Vo = torch.zeros_like(P), torch.zeros_like(P)
    loss = torch.zeros(1, device=dev)
    xt, yt, mt = (torch.from_numpy(a).to(dev) for a in (Xtr, Ytr, Mtr))
    g = np.random.default_rng(args.seed)
    t0 = time.time()
    hist = []
    for step in range(1, args.steps + 1):
        idx = torch.from_numpy(g.choice(ntr, size=min(args.batch, ntr), replace=False)).to(dev)
        xb, yb, mb = xt[idx].contiguous(), yt[idx].contiguous(), mt[idx].contiguous()
        valid = max(1.0, float(mb.sum().item()))
        st = L.gbblas_mlp_loss_grad(sb.handle, IN, HID, OUT, P.data_ptr(), xb.data_ptr(), yb.data_ptr(),
                                    mb.data_ptr(), len(idx), valid, G.data_ptr(), loss.data_ptr())
        assert st == 0, L.gbblas_last_error()
        lr = args.lr * (0.5 * (1 + np.cos(np.pi * step / args.steps)))  # cosine decay
        st = L.gbblas_mlp_adam(sb.handle, cnt.value, P.data_ptr(), G.data_ptr(), Mo.data_ptr(), Vo.data_ptr(), step,
                               float(lr), 0.9, 0.999, 1e-8, 1e-4)
        assert st == 0, L.gbblas_last_error()
        if step % 500 == 0 or step == 1:
            hist.append((step, float(loss.item())))
    torch.cuda.synchronize()
    train_s = time.time() - t0

    def predict(Xs):
        xs = torch.from_numpy(Xs).to(dev)
        ys = torch.empty(len(Xs), OUT, device=dev)
        st = L.gbblas_mlp_forward(sb.handle, IN, HID, OUT, P.data_ptr(), xs.data_ptr(), len(Xs), ys.data_ptr())
        assert st == 0, L.gbblas_last_error()
        return ys.cpu().numpy()

    pick_mlp = predict(Xte).argmin(1)
    pick_heur = np.array([L.gbblas_sgemm_heuristic_config(int(s[0]), int(s[1]), int(s[2]), int(s[3]))
                          for s in shapes[ntr:]])
    # best single fixed config (chosen on the training shapes)
    fixed = int(np.argmin(Ytr.mean(0)))  # mean clipped log2 slowdown over the training shapes
    pick_fixed = np.full(len(Xte), fixed)
    r_mlp, r_heur, r_fix = regret(Tte, pick_mlp), regret(Tte, pick_heur), regret(Tte, pick_fixed)
    tot_best = float(Tte.min(1).sum())
    report = {
        "train_shapes": int(ntr), "heldout_shapes": int(len(Xte)), "configs": OUT, "hidden": HID,
        "steps": args.steps, "batch": args.batch, "train_seconds": train_s, "loss_history": hist,
        "regret_mean": {"mlp": float(r_mlp.mean()), "heuristic": float(r_heur.mean()),
                        "best_fixed_config": float(r_fix.mean())},
        "regret_median": {"mlp": float(np.median(r_mlp)), "heuristic": float(np.median(r_heur))},
        "regret_p90": {"mlp": float(np.quantile(r_mlp, 0.9)), "heuristic": float(np.quantile(r_heur, 0.9))},
        "total_time_over_exhaustive": {
            "mlp": float(Tte[np.arange(len(Xte)), pick_mlp].sum() / tot_best),
            "heuristic": float(Tte[np.arange(len(Xte)), pick_heur].sum() / tot_best)},
        "exact_pick_rate_mlp": float((pick_mlp == Tte.argmin(1)).mean()),
        "best_fixed_config": fixed,
        "sweep_meta": json.loads(str(d["meta"])),
    }
    os.makedirs(args.out_dir, exist_ok=True)
    params = P.cpu().numpy()
    write_bin(os.path.join(args.out_dir, "sgemm_selector.bin"), params)
    with open(os.path.join(args.out_dir, "sgemm_selector_report.json"), "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps(report["regret_mean"]), json.dumps(report["total_time_over_exhaustive"]))


if __name__ == "__main__":
    main()
