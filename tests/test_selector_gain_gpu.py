"""What the trained selector gains over the method without it: on fresh
seeded shapes (not in the training sweep), every config is timed
exhaustively and the regret t(pick)/t(best) - 1 of the learned selector is
compared with that of the fixed size-threshold heuristic."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_learned_selector_beats_heuristic(sb, torch_cuda):
    torch = torch_cuda
    from portblas_gb300 import _lib
    from portblas_gb300.tuning import sweep
    L = _lib.load()
    shapes = sweep.sample_shapes(24, seed=555)
    A = torch.rand(sweep.ELEM_CAP + 4096, device="cuda")
    B = torch.rand(sweep.ELEM_CAP + 4096, device="cuda")
    Cm = torch.zeros(sweep.ELEM_CAP + 65536, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r_mlp, r_heur = [], []
    for s in shapes:
        m, n, k = s["m"], s["n"], s["k"]
        sa = (m * s["lda"]) if s["ta"] else (k * s["lda"])
        sbs = (k * s["ldb"]) if s["tb"] else (n * s["ldb"])
        sc = n * s["ldc"]
        bt = max(1, min(s["batch"], (sweep.ELEM_CAP + 4096) // max(sa, sbs, sc)))
        ta, tb = (b"t" if s["ta"] else b"n"), (b"t" if s["tb"] else b"n")
        t = np.full(40, np.inf)
        for c in range(40):
            run = lambda: L.gbblas_sgemm_strided_batched_config(sb.handle, c, ta, tb, m, n, k, 1.0, A.data_ptr(),
                                                                s["lda"], sa, B.data_ptr(), s["ldb"], sbs, 0.0,
                                                                Cm.data_ptr(), s["ldc"], sc, bt)
            if run() != 0:
                continue
            e0.record()
            for _ in range(3):
                run()
            e1.record()
            e1.synchronize()
            t[c] = e0.elapsed_time(e1) / 3
        pick = C.c_int()
        assert L.gbblas_sgemm_selector_pick(m, n, k, ta, tb, s["lda"], s["ldb"], s["ldc"], bt, C.byref(pick)) == 0
        r_mlp.append(t[pick.value] / t.min() - 1)
        r_heur.append(t[L.gbblas_sgemm_heuristic_config(m, n, k, bt)] / t.min() - 1)
    assert np.mean(r_mlp) < np.mean(r_heur), (np.mean(r_mlp), np.mean(r_heur))
    assert np.mean(r_mlp) <= 0.15, r_mlp
