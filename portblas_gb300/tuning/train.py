"""Trains the GEMM tile selector on a sweep's timing table with the
library's own CUDA kernels (gbblas_mlp_loss_grad / gbblas_mlp_adam), then
measures its regret against exhaustive autotuning on held-out shapes, per
element type.

Target: for each shape and config, log2(t_config / t_best), clipped at 8
(configs that cannot run, or belong to the other element type, are masked
out).  Selection = argmin of the predicted targets over the shape's element
type's configs.  Regret of a selector on a shape = t(pick)/t(best) - 1.

Run on a GPU:
  python -m portblas_gb300.tuning.train --sweep FILE.npz --out-dir DIR
writes DIR/gemm_selector.bin (the weights the library loads) and
DIR/gemm_selector_report.json.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import struct
import time

import numpy as np

IN, HID, OUT = 11, 64, 60
F64_FIRST = 40  # FP32 configs [0, 40), FP64 configs [40, 60)
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
    dt = d["dtype"][keep] if "dtype" in d.files else np.zeros(len(X), np.int8)
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

    def pick_in_range(pred, is64):
        lo = np.where(is64, F64_FIRST, 0)
        hi = np.where(is64, OUT, F64_FIRST)
        col = np.arange(OUT)[None, :]
        masked = np.where((col >= lo[:, None]) & (col < hi[:, None]), pred, np.inf)
        return masked.argmin(1)

    is64_tr, is64_te = dt[:ntr] == 1, dt[ntr:] == 1
    pick_mlp = pick_in_range(predict(Xte), is64_te)
    pick_heur = np.array([L.gbblas_gemm_heuristic_config(2 if f64 else 0, int(s[0]), int(s[1]), int(s[2]),
                                                         int(s[3]))
                          for s, f64 in zip(shapes[ntr:], is64_te)])
    # best single fixed config per element type (chosen on the training shapes)
    fixed = {}
    for name, sel, lo, hi in (("f32", ~is64_tr, 0, F64_FIRST), ("f64", is64_tr, F64_FIRST, OUT)):
        fixed[name] = lo + int(np.argmin(Ytr[sel][:, lo:hi].mean(0))) if sel.any() else lo
    pick_fixed = np.where(is64_te, fixed["f64"], fixed["f32"])
    r_mlp, r_heur, r_fix = regret(Tte, pick_mlp), regret(Tte, pick_heur), regret(Tte, pick_fixed)

    def summary(sel):
        if not sel.any():
            return None
        tb = float(Tte[sel].min(1).sum())
        idx = np.flatnonzero(sel)
        return {
            "heldout_shapes": int(sel.sum()),
            "regret_mean": {"mlp": float(r_mlp[sel].mean()), "heuristic": float(r_heur[sel].mean()),
                            "best_fixed_config": float(r_fix[sel].mean())},
            "regret_median": {"mlp": float(np.median(r_mlp[sel])), "heuristic": float(np.median(r_heur[sel]))},
            "regret_p90": {"mlp": float(np.quantile(r_mlp[sel], 0.9)),
                           "heuristic": float(np.quantile(r_heur[sel], 0.9))},
            "total_time_over_exhaustive": {"mlp": float(Tte[idx, pick_mlp[sel]].sum() / tb),
                                           "heuristic": float(Tte[idx, pick_heur[sel]].sum() / tb)},
            "exact_pick_rate_mlp": float((pick_mlp[sel] == Tte[sel].argmin(1)).mean()),
        }

    all_te = np.ones(len(Xte), dtype=bool)
    report = {
        "train_shapes": int(ntr), "configs": OUT, "hidden": HID,
        "steps": args.steps, "batch": args.batch, "train_seconds": train_s, "loss_history": hist,
        **summary(all_te),
        "per_dtype": {"f32": summary(~is64_te), "f64": summary(is64_te)},
        "best_fixed_config": fixed,
        "sweep_meta": json.loads(str(d["meta"])),
    }
    os.makedirs(args.out_dir, exist_ok=True)
    params = P.cpu().numpy()
    write_bin(os.path.join(args.out_dir, "gemm_selector.bin"), params)
    with open(os.path.join(args.out_dir, "gemm_selector_report.json"), "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps(report["regret_mean"]), json.dumps(report["total_time_over_exhaustive"]),
          json.dumps({k: v and v["regret_mean"] for k, v in report["per_dtype"].items()}))


if __name__ == "__main__":
    main()
