"""Learned element preconditioner on the GPU: forward and gradient against the
oracle's 3D-convolution / GELU restatement (composed as in tests/test_oracle.py,
whose composition is itself checked by finite differences), training progress,
checkpoint round trip, and its use inside flexible PCG.

Tolerances: forward 2e-5 relative (BF16 weights are used for inference, so the
oracle is fed the BF16-rounded weights); gradient 1e-4 relative (FP32)."""
import os

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
_net_forward = oracle.net_forward
net_loss_grad = oracle.net_loss_grad


def bf16(w):
    f = np.asarray(w, np.float32).view(np.uint32).astype(np.uint64)
    lsb = (f >> 16) & 1
    return (((f + 0x7FFF + lsb) >> 16) << 16).astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("Nq,C", [(4, 8), (8, 16), (6, 16)])
def test_forward_matches_oracle(nb, O, dev, Nq, C):
    E = 5
    net = nb.Net(Nq, C, 3, seed=3)
    W = net.weights()
    x = O.uniform(E * Nq ** 3, 4, 1, -1, 1).astype(np.float32)
    out = torch.zeros(E * Nq ** 3, dtype=torch.float32, device=dev)
    net.forward(torch.from_numpy(x).to(dev), out, E)
    torch.cuda.synchronize()
    ref, _ = _net_forward(Nq, bf16(W), x, C)
    got = out.cpu().numpy()
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()


@pytest.mark.parametrize("Nq,C,E", [(4, 8, 7), (8, 16, 3)])
def test_gradient_matches_oracle(nb, O, dev, Nq, C, E):
    net = nb.Net(Nq, C, 3, seed=5)
    rng = np.random.default_rng(2)
    W = (rng.standard_normal(net.P) * 0.3).astype(np.float32)
    net.set_weights(W)
    x = rng.standard_normal(E * Nq ** 3).astype(np.float32)
    t = rng.standard_normal(E * Nq ** 3).astype(np.float32)
    g, loss = net.gradient(torch.from_numpy(x).to(dev), torch.from_numpy(t).to(dev), E)
    loss_ref, g_ref = net_loss_grad(Nq, W, x, t, C)
    assert abs(loss - loss_ref) <= 1e-5 * loss_ref
    assert np.abs(g - g_ref).max() <= 1e-4 * np.abs(g_ref).max()
    # deterministic reduction: identical bits on a second call
    g2, loss2 = net.gradient(torch.from_numpy(x).to(dev), torch.from_numpy(t).to(dev), E)
    assert np.array_equal(g, g2) and loss == loss2


def test_training_fits_a_local_linear_map(nb, O, dev):
    """The network learns t = (discrete Laplacian smoothing of x) on element blocks."""
    Nq, C, E = 4, 8, 512
    net = nb.Net(Nq, C, 3, seed=7)
    rng = np.random.default_rng(3)
    x = rng.standard_normal((E, Nq, Nq, Nq)).astype(np.float32)
    t = x.copy()
    t[:, 1:-1, 1:-1, 1:-1] = 0.5 * x[:, 1:-1, 1:-1, 1:-1] + 0.25 * (
        x[:, 2:, 1:-1, 1:-1] + x[:, :-2, 1:-1, 1:-1])
    xd = torch.from_numpy(x.ravel()).to(dev)
    td = torch.from_numpy(t.ravel()).to(dev)
    losses = [net.train_step(xd, td, E, 3e-3) for _ in range(300)]
    assert losses[-1] < 0.2 * losses[0]


def test_checkpoint_round_trip(nb, dev, tmp_path):
    net = nb.Net(8, 16, 3, seed=9)
    x = torch.randn(2 * 512, device=dev)
    net.train_step(x, x, 2, 1e-3)
    path = os.path.join(tmp_path, "net.bin")
    net.save(path)
    net2 = nb.Net.load(path)
    assert np.array_equal(net.weights(), net2.weights())
    # both continue identically (Adam moments and step restored)
    l1 = net.train_step(x, x, 2, 1e-3)
    l2 = net2.train_step(x, x, 2, 1e-3)
    assert l1 == l2 and np.array_equal(net.weights(), net2.weights())
    # a damaged file is rejected
    raw = bytearray(open(path, "rb").read())
    raw[100] ^= 0xFF
    open(path, "wb").write(bytes(raw))
    with pytest.raises(nb.NekbError):
        nb.Net.load(path)


def test_flexible_pcg_with_network_converges(nb, O, dev):
    """The untrained network (near-zero last layer) leaves Jacobi-FPCG intact; the
    solve reaches the FP64 tolerance through the learned-preconditioner path."""
    bp = nb.BP(7, 4, 4, 4, perturb=0.1, seed=3)
    L = bp.Nlocal
    lam = torch.cat([torch.full((L,), 1.0), torch.full((L,), 1.5)]).double().to(dev)
    f = torch.from_numpy(O.uniform(L, 8, 3, -1, 1)).to(dev)
    bp.ogs.gather_scatter_many(f)
    net = nb.Net(8, 16, 3, seed=11)
    r, x = f.clone(), torch.zeros_like(f)
    st = bp.pcg(lam, r, x, 1e-8, 2000, solver=nb.SOLVER_MIXED, precond=nb.PRECOND_LEARNED, net=net)
    assert st["status"] == 0 and st["true_rel_res"] <= 1e-8
    r2, x2 = f.clone(), torch.zeros_like(f)
    st2 = bp.pcg(lam, r2, x2, 1e-8, 2000, solver=nb.SOLVER_MIXED)
    assert float((x - x2).abs().max() / x2.abs().max()) < 1e-6
