"""The selector's CUDA training kernels against the FP64 oracle
(oracle/mlp.py): forward values, loss and every gradient, one AdamW step,
and run-to-run determinism."""
import ctypes as C

import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu
IN, HID, OUT = 11, 64, 60


@pytest.fixture(scope="module")
def L(torch_cuda):
    from portblas_gb300 import _lib, build
    build.build()
    return _lib.load()


def _setup(torch, n=300, seed=0):
    from portblas_gb300.tuning import train
    g = np.random.default_rng(seed)
    p = train.init_params(seed)
    x = g.random((n, IN)).astype(np.float32)
    t = (g.random((n, OUT)) * 4).astype(np.float32)
    m = (g.random((n, OUT)) < 0.9).astype(np.float32)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return p, x, t, m, dev


def test_forward_matches_oracle(sb, L, torch_cuda):
    torch = torch_cuda
    p, x, t, m, dev = _setup(torch)
    y = torch.empty(len(x), OUT, device="cuda")
    P, X = dev(p), dev(x)
    assert L.gbblas_mlp_forward(sb.handle, IN, HID, OUT, P.data_ptr(), X.data_ptr(), len(x), y.data_ptr()) == 0
    ref, _, _ = omlp.forward(p, x, IN, HID, OUT)
    np.testing.assert_allclose(y.cpu().numpy(), ref, rtol=1e-4, atol=1e-4)


def test_gradients_match_oracle(sb, L, torch_cuda):
    torch = torch_cuda
    p, x, t, m, dev = _setup(torch, seed=1)
    P, X, T, M = dev(p), dev(x), dev(t), dev(m)
    G = torch.zeros_like(P)
    loss = torch.zeros(1, device="cuda")
    valid = float(m.sum())
    assert L.gbblas_mlp_loss_grad(sb.handle, IN, HID, OUT, P.data_ptr(), X.data_ptr(), T.data_ptr(), M.data_ptr(),
                                  len(x), valid, G.data_ptr(), loss.data_ptr()) == 0
    ref_loss, ref_g = omlp.loss_grad(p, x, t, m, IN, HID, OUT, valid)
    assert abs(loss.item() - ref_loss) <= 1e-4 * abs(ref_loss)
    got = G.cpu().numpy()
    scale = np.abs(ref_g).max()
    np.testing.assert_allclose(got, ref_g, rtol=1e-3, atol=1e-4 * scale)
    # determinism: a second evaluation is bit-identical
    G2 = torch.zeros_like(P)
    L.gbblas_mlp_loss_grad(sb.handle, IN, HID, OUT, P.data_ptr(), X.data_ptr(), T.data_ptr(), M.data_ptr(), len(x),
                           valid, G2.data_ptr(), loss.data_ptr())
    assert torch.equal(G, G2)


def test_adam_step_matches_definition(sb, L, torch_cuda):
    torch = torch_cuda
    g = np.random.default_rng(2)
    n = 1000
    p, gr = g.standard_normal(n).astype(np.float32), g.standard_normal(n).astype(np.float32)
    m0, v0 = g.standard_normal(n).astype(np.float32), g.random(n).astype(np.float32)
    P, Gd, Md, Vd = (torch.from_numpy(a.copy()).cuda() for a in (p, gr, m0, v0))
    lr, b1, b2, eps, wd, step = 1e-3, 0.9, 0.999, 1e-8, 1e-4, 3
    assert L.gbblas_mlp_adam(sb.handle, n, P.data_ptr(), Gd.data_ptr(), Md.data_ptr(), Vd.data_ptr(), step, lr, b1, b2,
                             eps, wd) == 0
    m1 = b1 * m0 + (1 - b1) * gr
    v1 = b2 * v0 + (1 - b2) * gr * gr
    ref = p - lr * ((m1 / (1 - b1 ** step)) / (np.sqrt(v1 / (1 - b2 ** step)) + eps) + wd * p)
    np.testing.assert_allclose(P.cpu().numpy(), ref, rtol=1e-5, atol=1e-6)
