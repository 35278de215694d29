"""The learned tuner's MLP: the FP64 oracle is pinned by finite differences
(CPU), and the CUDA forward / backward / MSE / Adam kernels (through the C
ABI) match it (GPU)."""
import ctypes

import numpy as np
import pytest

import oracle.mlp as om

D = 24


def rand_problem(B=300, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(B, D)).astype(np.float32)
    P = (rng.normal(size=D * 64 + 64 + 64 * 64 + 64 + 64 + 1) * 0.2).astype(np.float32)
    dY = rng.normal(size=B).astype(np.float32)
    return X, P, dY


def test_oracle_gradients_match_finite_differences():
    X, P, dY = rand_problem(B=40)
    rng = np.random.default_rng(3)
    idx = rng.choice(P.size, 60, replace=False)
    for fd, an in om.check_gradients_fd(X, P.astype(np.float64), D, dY.astype(np.float64), idx):
        assert abs(fd - an) <= 1e-5 * max(1.0, abs(an)), (fd, an)


@pytest.mark.gpu
def test_cuda_forward_backward_match_fp64_oracle():
    import torch

    from kokkos_gb300 import gbk
    X, P, dY = rand_problem()
    B = X.shape[0]
    assert gbk.lib.gbk_mlp_param_count(D) == P.size
    Xd, Pd, dYd = (torch.from_numpy(a).cuda() for a in (X, P, dY))
    acts = torch.empty(B * 128, dtype=torch.float32, device="cuda")
    Y = torch.empty(B, dtype=torch.float32, device="cuda")
    G = torch.empty_like(Pd)
    p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    gbk.check(gbk.lib.gbk_mlp_forward(p(Xd), B, D, p(Pd), p(acts), p(Y), None))
    gbk.check(gbk.lib.gbk_mlp_backward(p(Xd), B, D, p(Pd), p(acts), p(dYd), p(G), None))
    torch.cuda.synchronize()
    Yw, A1, A2 = om.forward(X, P, D)
    np.testing.assert_allclose(Y.cpu().numpy(), Yw, rtol=1e-4, atol=1e-4)
    a = acts.cpu().numpy().reshape(B, 128)
    np.testing.assert_allclose(a[:, :64], A1, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(a[:, 64:], A2, rtol=1e-4, atol=1e-5)
    gw = om.backward(X, P, D, dY)
    g = G.cpu().numpy()
    # per parameter block, relative to the block's norm (FP32 accumulation)
    o = 0
    for sz in (D * 64, 64, 64 * 64, 64, 64, 1):
        gb, wb = g[o:o + sz], gw[o:o + sz]
        assert np.linalg.norm(gb - wb) <= 1e-4 * max(np.linalg.norm(wb), 1e-6), (o, sz)
        o += sz


@pytest.mark.gpu
def test_cuda_mse_and_adam_step():
    import torch

    from kokkos_gb300 import gbk
    rng = np.random.default_rng(1)
    B, P = 1000, 777
    Y, T = rng.normal(size=B).astype(np.float32), rng.normal(size=B).astype(np.float32)
    Yd, Td = torch.from_numpy(Y).cuda(), torch.from_numpy(T).cuda()
    dY = torch.empty(B, device="cuda")
    loss = torch.zeros(1, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    gbk.check(gbk.lib.gbk_mlp_mse(p(Yd), p(Td), B, p(dY), p(loss), None))
    lw, dw = om.mse(Y, T)
    assert abs(loss.item() - lw) <= 1e-5 * lw
    np.testing.assert_allclose(dY.cpu().numpy(), dw, rtol=1e-5, atol=1e-8)
    w = rng.normal(size=P).astype(np.float32)
    g = rng.normal(size=P).astype(np.float32)
    wd, gd = torch.from_numpy(w.copy()).cuda(), torch.from_numpy(g).cuda()
    m, v = torch.zeros(P, device="cuda"), torch.zeros(P, device="cuda")
    gbk.check(gbk.lib.gbk_mlp_adam(p(wd), p(gd), p(m), p(v), P, 1e-2, 0.9, 0.999, 1e-8, 1, None))
    mh = (0.1 * g) / (1 - 0.9)
    vh = (0.001 * g * g) / (1 - 0.999)
    np.testing.assert_allclose(wd.cpu().numpy(), w - 1e-2 * mh / (np.sqrt(vh) + 1e-8), rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
def test_training_fits_a_smooth_function():
    from kokkos_gb300.tuner import MLP
    rng = np.random.default_rng(2)
    X = rng.uniform(-1, 1, size=(6000, D)).astype(np.float32)
    T = np.sin(2 * X[:, 0]) + X[:, 1] * X[:, 2] + 0.5 * np.abs(X[:, 3])
    m = MLP(D=D, seed=0)
    hist = m.train(X, T, epochs=150, batch=1024, lr=3e-3)
    assert hist[-1][1] < 0.1 * hist[0][1], hist
    pred = m.predict(X[:500])
    assert np.sqrt(np.mean((pred - T[:500]) ** 2)) < 0.25 * np.std(T)
