"""Learned warm start: the MLP kernels' gradients against the CPU oracle, a
training run that drives the loss down, and a warm-started sweep that reaches
the same steady state as the standard initial condition in fewer steps."""
import numpy as np
import pytest

import pecs_gb300 as pg
from oracle import nn_oracle

pytestmark = pytest.mark.gpu


def _torch():
    return pytest.importorskip("torch")


def test_mlp_gradients_match_cpu_oracle(pecs_lib):
    torch = _torch()
    from pecs_gb300.learned import Mlp
    widths = [6, 64, 48, 10]
    m = Mlp(widths, seed=3)
    rng = np.random.default_rng(0)
    p = rng.standard_normal(m.n_params).astype(np.float32) * 0.2
    m.set_params(p)
    x = rng.uniform(-1, 1, (32, 6)).astype(np.float32)
    t = rng.standard_normal((32, 10)).astype(np.float32)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    g, loss = m.gradients(xd.data_ptr(), td.data_ptr(), 32)
    loss_ref, g_ref = nn_oracle.loss_and_grad(p, widths, x, t)
    assert abs(loss - loss_ref) <= 1e-4 * abs(loss_ref)
    assert np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref) < 2e-3
    # forward agrees with the oracle too
    y = torch.empty(32, 10, device="cuda")
    m.forward(xd.data_ptr(), y.data_ptr(), 32)
    y_ref = nn_oracle.forward(p, widths, x)[-1]
    assert np.max(np.abs(y.cpu().numpy() - y_ref)) < 1e-3 * np.max(np.abs(y_ref))


def test_mlp_tensor_core_gemms_across_tiles(pecs_lib):
    """Widths and batch that are not multiples of the tensor-core tile (128 x
    128, K chunks of 64): several tiles and chunks per GEMM, ragged edges in
    M, N and K, for the forward GEMM and both backward GEMMs."""
    torch = _torch()
    from pecs_gb300.learned import Mlp
    widths = [6, 200, 300, 70]
    m = Mlp(widths, seed=4)
    rng = np.random.default_rng(1)
    p = (rng.standard_normal(m.n_params) * 0.1).astype(np.float32)
    m.set_params(p)
    B = 150
    x = rng.uniform(-1, 1, (B, 6)).astype(np.float32)
    t = rng.standard_normal((B, 70)).astype(np.float32)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    y = torch.empty(B, 70, device="cuda")
    m.forward(xd.data_ptr(), y.data_ptr(), B)
    y_ref = nn_oracle.forward(p, widths, x)[-1]
    assert np.max(np.abs(y.cpu().numpy() - y_ref)) < 1e-3 * np.max(np.abs(y_ref))
    g, loss = m.gradients(xd.data_ptr(), td.data_ptr(), B)
    loss_ref, g_ref = nn_oracle.loss_and_grad(p, widths, x, t)
    assert abs(loss - loss_ref) <= 1e-4 * abs(loss_ref)
    assert np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref) < 2e-3


def test_mlp_training_reduces_loss(pecs_lib):
    torch = _torch()
    from pecs_gb300.learned import Mlp
    m = Mlp([6, 128, 128, 4], seed=1)
    x = torch.rand(512, 6, device="cuda") * 2 - 1
    t = torch.stack([x[:, 0] * x[:, 1], torch.sin(2 * x[:, 2]), x[:, 3] ** 2, x[:, 4] - x[:, 5]], 1)
    first = m.train_step(x.data_ptr(), t.contiguous().data_ptr(), 512, 3e-3, want_loss=True)
    for _ in range(400):
        last = m.train_step(x.data_ptr(), t.contiguous().data_ptr(), 512, 3e-3, want_loss=True)
    assert last < 0.1 * first


def test_warm_start_saves_steps_and_keeps_the_steady_state(pecs_lib):
    torch = _torch()
    from pecs_gb300 import learned as L
    base = pg.half_cell(n_refine=3)
    thetas = L.sample(96, seed=5)
    tr, ev = thetas[:64], thetas[64:]
    ctx = pg.Context([L.instance_params(t, base) for t in tr[:32]], precision=pg.PREC_FP32_MIXED)
    lay = L.Layout.of(ctx)
    Y, steps_tr = L.steady_states(ctx, tr, base)
    op = L.NeuralOperator(rank=16, hidden=128, seed=0)
    T = op.fit_basis(Y, lay)
    X = torch.from_numpy(L.normalize(tr)).cuda()
    hist = op.train(X, T, epochs=300, batch=32, lr=2e-3)
    assert hist[-1] < 0.2 * hist[0]
    # the fused library kernel (decode, exp, scatter) against the decode + torch
    Xe = torch.from_numpy(L.normalize(ev)).cuda()
    vn, vp = op.predict_vectors(Xe, lay)
    y = op.predict(Xe)
    u = slice(lay.u_off, lay.u_off + lay.n_u)
    assert torch.allclose(vn[:, u], y[:, :lay.n_u].exp(), rtol=1e-5, atol=0)
    assert torch.allclose(vp[:, u], y[:, lay.n_u:2 * lay.n_u].exp(), rtol=1e-5, atol=0)
    assert (vn[:, :lay.u_off] == 0).all() and (vp[:, :lay.u_off] == 0).all()
    s_w, fb, c_w = L.warm_started_sweep(ctx, op, ev, base)
    s_p, _, c_p = L.warm_started_sweep(ctx, None, ev, base)
    assert s_w.sum() < s_p.sum()                      # fewer steps overall
    assert np.max(np.abs(c_w - c_p) / np.abs(c_p)) < 1e-5   # same steady-state current
