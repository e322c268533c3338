"""Learned element preconditioner on the GPU: forward and gradient against the
oracle's 3D-convolution / GELU restatement (composed as in tests/test_oracle.py,
whose composition is itself checked by finite differences), training progress,
checkpoint round trip, and its use inside flexible PCG.

Tolerances: FP32-core forward 2e-5 relative (BF16 weights are used for
inference, so the oracle is fed the BF16-rounded weights); tensor-core forward
1e-2 of the output's max-norm and 2e-3 in RMS (the oracle rounds the input and
both GELU outputs to BF16 as the kernel does; a different FP32 summation order
or the hardware tanh can move an activation by one BF16 step); gradient 1e-4
relative (FP32)."""
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
    net.inference = nb.NET_FP32
    assert net.inference == nb.NET_FP32
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


@pytest.mark.parametrize("N", [3, 7])
def test_local_correction_is_the_element_interior_solve(nb, O, dev, N):
    """nekb_bp_local_correction against a dense solve of each element's
    interior block, the element matrix assembled column by column from the
    oracle's axhelm; Jacobi values on the element boundary; a row whose element
    index is outside the mesh comes back zero.  Tolerance 1e-3 relative (FP32 CG
    to a relative residual of 1e-6)."""
    Nq = N + 1
    Np = Nq ** 3
    bp = nb.BP(N, 2, 2, 2, perturb=0.15, seed=5)
    E, L = bp.E, bp.Nlocal
    lam = np.concatenate([0.5 + O.uniform(L, 21, 1), 1.0 + O.uniform(L, 21, 2)])
    lam_d = torch.from_numpy(lam).to(dev)
    elems = np.array([0, 5, 7, 3, E], dtype=np.int32)
    n = len(elems)
    r = O.uniform(n * Np, 22, 1, -1, 1).astype(np.float32)
    dinv = (0.1 + O.uniform(n * Np, 22, 2)).astype(np.float32)
    y = torch.full((n * Np,), 7.0, dtype=torch.float32, device=dev)
    bp.local_correction(lam_d, torch.from_numpy(elems).to(dev), torch.from_numpy(r).to(dev),
                        torch.from_numpy(dinv).to(dev), y, iters=500, tol=1e-6)
    torch.cuda.synchronize()
    got = y.cpu().numpy().reshape(n, Np)
    ggeo = bp.device_array("ggeo", 7 * L, torch.float64).cpu().numpy()
    D = O.dmatrix(O.gll(N)[0])
    ii = np.arange(Nq)
    I3 = np.stack(np.meshgrid(ii, ii, ii, indexing="ij"), -1).reshape(-1, 3)[:, ::-1]  # (i,j,k)
    interior = np.all((I3 > 0) & (I3 < N), axis=1)
    for b, e in enumerate(elems[:-1]):
        ge = ggeo[e * 7 * Np:(e + 1) * 7 * Np]
        le = np.concatenate([lam[e * Np:(e + 1) * Np], lam[L + e * Np:L + (e + 1) * Np]])
        A = np.stack([O.axhelm(Nq, 1, Np, 0, ge, D, le, np.eye(Np)[c]) for c in range(Np)], 1)
        rb = r[b * Np:(b + 1) * Np].astype(np.float64)
        want = dinv[b * Np:(b + 1) * Np] * rb
        want[interior] = np.linalg.solve(A[np.ix_(interior, interior)], rb[interior])
        assert np.abs(got[b] - want).max() <= 1e-3 * np.abs(want).max(), (N, b)
    assert np.all(got[-1] == 0.0)


@pytest.mark.parametrize("mode", ["NET_TENSOR", "NET_TENSOR_SYNC", "NET_TENSOR_TC5"])
@pytest.mark.parametrize("seed", [3, 4])
def test_tensor_core_forward_matches_oracle(nb, O, dev, seed, mode):
    """Every tensor-core kernel (the default, warp-level mma.sync, and tcgen05
    with accumulators in tensor memory) against the oracle's convolutions on
    BF16-rounded weights and activations; E = 37 elements, so the persistent
    grid's CTAs take different element counts."""
    Nq, C, E = 8, 16, 37
    net = nb.Net(Nq, C, 3, seed=seed)
    assert net.inference == nb.NET_TENSOR
    net.inference = getattr(nb, mode)
    assert net.inference == getattr(nb, mode)
    W = bf16(net.weights())
    x = O.uniform(E * Nq ** 3, 40 + seed, 1, -1, 1).astype(np.float32)
    out = torch.zeros(E * Nq ** 3, dtype=torch.float32, device=dev)
    net.forward(torch.from_numpy(x).to(dev), out, E)
    torch.cuda.synchronize()
    o2, o3 = 27 * C, 27 * C + 27 * C * C
    a1 = bf16(O.gelu(O.conv3d_forward(Nq, W[:o2], bf16(x), 1, C)))
    a2 = bf16(O.gelu(O.conv3d_forward(Nq, W[o2:o3], a1, C, C)))
    ref = O.conv3d_forward(Nq, W[o3:], a2, C, 1).astype(np.float64)
    d = out.cpu().numpy().astype(np.float64) - ref
    assert np.abs(d).max() <= 1e-2 * np.abs(ref).max()
    assert np.sqrt(np.mean(d * d)) <= 2e-3 * np.sqrt(np.mean(ref * ref))


def test_tensor_core_kernels_agree_on_many_elements(nb, O, dev):
    """tcgen05 and mma.sync inference on 3000 elements (each CTA of the
    persistent grids loops over several elements), with the solver's input
    scaling, Jacobi term and weights: the same BF16 arithmetic in different
    summation orders, so the outputs agree to a few BF16 steps of the
    activations."""
    net = nb.Net(8, 16, 3, seed=9)
    E = 3000
    x = torch.from_numpy(O.uniform(E * 512, 77, 1, -1, 1).astype(np.float32)).to(dev)
    outs = []
    for mode in (nb.NET_TENSOR_TC5, nb.NET_TENSOR_SYNC):
        net.inference = mode
        o = torch.zeros_like(x)
        net.forward(x, o, E)
        outs.append(o)
    torch.cuda.synchronize()
    d = (outs[0] - outs[1]).double()
    ref = outs[1].double()
    assert float(d.abs().max()) <= 1e-2 * float(ref.abs().max())
    assert float(d.pow(2).mean().sqrt()) <= 2e-3 * float(ref.pow(2).mean().sqrt())


def test_learned_solve_on_tcgen05_kernel(nb, O, dev):
    """Flexible CG with the network evaluated by the tcgen05 kernel reaches the
    FP64 tolerance and takes about the iterations of the mma.sync kernel."""
    bp = nb.BP(7, 6, 6, 6, perturb=0.1, seed=3)
    L = bp.Nlocal
    lam = torch.cat([torch.full((L,), 1.0), torch.full((L,), 1.5)]).double().to(dev)
    f = torch.from_numpy(O.uniform(L, 8, 3, -1, 1)).to(dev)
    bp.ogs.gather_scatter_many(f)
    net = nb.Net.load(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                   "nekbench_gb300", "weights", "precond_n7_c16.bin"))
    its = {}
    for mode in (nb.NET_TENSOR_TC5, nb.NET_TENSOR_SYNC):
        net.inference = mode
        r, x = f.clone(), torch.zeros_like(f)
        st = bp.pcg(lam, r, x, 1e-8, 3000, solver=nb.SOLVER_MIXED, precond=nb.PRECOND_LEARNED,
                    net=net)
        assert st["status"] == 0 and st["true_rel_res"] <= 1e-8
        its[mode] = st["iterations"]
    assert abs(its[nb.NET_TENSOR_TC5] - its[nb.NET_TENSOR_SYNC]) <= 0.1 * its[nb.NET_TENSOR_SYNC] + 5, its


def test_captured_solver_graph_follows_the_network(nb, O, dev):
    """The solver replays one captured CUDA graph per chunk of iterations and
    keeps it for the next solve with the same arguments.  A solve on the same
    problem and buffers with another network, or with the same network on the
    other inference kernel, runs that network: its iterates equal those of a
    fresh problem object that never saw the first network."""
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "nekbench_gb300", "weights", "precond_n7_c16.bin")
    trained = nb.Net.load(path)
    other = nb.Net.load(path)
    w = np.asarray(other.weights(), np.float32).copy()
    w[27 * 16:] *= -0.5  # another network: layers 2 and 3 changed
    other.set_weights(w)

    def make():
        bp = nb.BP(7, 3, 3, 3, perturb=0.1, seed=3)
        L = bp.Nlocal
        lam = torch.cat([torch.full((L,), 1.0), torch.full((L,), 1.5)]).double().to(dev)
        f = torch.from_numpy(O.uniform(L, 8, 3, -1, 1)).to(dev)
        bp.ogs.gather_scatter_many(f)
        return bp, lam, f

    def solve(bp, lam, f, r, x, net, mode):
        net.inference = mode
        r.copy_(f)
        x.zero_()
        bp.pcg(lam, r, x, 1e-12, 24, solver=nb.SOLVER_MIXED, precond=nb.PRECOND_LEARNED, net=net,
               fixed_iterations=True)
        torch.cuda.synchronize()
        return x.clone()

    bp, lam, f = make()
    r, x = torch.empty_like(f), torch.empty_like(f)
    runs = [(trained, nb.NET_TENSOR_TC5), (other, nb.NET_TENSOR_TC5), (trained, nb.NET_TENSOR_SYNC),
            (trained, nb.NET_FP32)]
    shared = [solve(bp, lam, f, r, x, net, mode) for net, mode in runs]
    for (net, mode), got in zip(runs, shared):
        bp2, lam2, f2 = make()
        want = solve(bp2, lam2, f2, torch.empty_like(f2), torch.empty_like(f2), net, mode)
        assert torch.equal(got, want), (mode, float((got - want).abs().max()))
    # the runs differ from one another, so a replayed graph would have shown
    assert not torch.equal(shared[0], shared[1])
    assert not torch.equal(shared[0], shared[3])


def test_inference_mode_falls_back_where_not_built(nb):
    net = nb.Net(4, 8, 3, seed=1)
    assert net.inference == nb.NET_FP32
    net.inference = nb.NET_TENSOR
    assert net.inference == nb.NET_FP32
    with pytest.raises(nb.NekbError):
        net.inference = 7


def test_fcg_window_with_a_zero_network_matches_jacobi(nb, O, dev):
    """A network whose last layer is zero adds nothing to Jacobi: FCG(m) for
    m = 1, 5, 8 (ring of kept directions, fused projections) is then PCG with
    Jacobi in exact arithmetic, so it takes the Jacobi-PCG count within a few
    iterations and reaches the FP64 tolerance; m = 9 is refused."""
    bp = nb.BP(7, 4, 4, 4, perturb=0.1, seed=3)
    L = bp.Nlocal
    lam = torch.cat([torch.full((L,), 1.0), torch.full((L,), 1.5)]).double().to(dev)
    f = torch.from_numpy(O.uniform(L, 8, 3, -1, 1)).to(dev)
    bp.ogs.gather_scatter_many(f)
    r, x = f.clone(), torch.zeros_like(f)
    jac = bp.pcg(lam, r, x, 1e-8, 2000, solver=nb.SOLVER_MIXED)
    net = nb.Net(8, 16, 3, seed=11)
    W = net.weights()
    W[27 * 16 + 27 * 16 * 16:] = 0.0
    net.set_weights(W)
    for m in (1, 5, 8):
        r, x = f.clone(), torch.zeros_like(f)
        st = bp.pcg(lam, r, x, 1e-8, 2000, solver=nb.SOLVER_MIXED, precond=nb.PRECOND_LEARNED,
                    net=net, fcg_window=m)
        assert st["status"] == 0 and st["true_rel_res"] <= 1e-8
        assert abs(st["iterations"] - jac["iterations"]) <= 3, (m, st, jac)
    with pytest.raises(nb.NekbError):
        bp.pcg(lam, f.clone(), torch.zeros_like(f), 1e-8, 10, solver=nb.SOLVER_MIXED,
               precond=nb.PRECOND_LEARNED, net=net, fcg_window=9)


def test_copy_timeout_flag_becomes_an_error_status(nb, O, dev):
    """The tensor-core kernel's bounded wait on its bulk input copies ends, if
    the copies never arrive, by raising a device flag; the host turns the flag
    into NEKB_ERR_CUDA.  Here the flag is raised from the host (no device wait
    runs out): the next forward and the next learned solve report the error,
    each clears the flag, and the call after it succeeds."""
    net = nb.Net(8, 16, 3, seed=5)
    assert net.inference == nb.NET_TENSOR
    E = 4
    x = torch.from_numpy(O.uniform(E * 512, 15, 1, -1, 1).astype(np.float32)).to(dev)
    out = torch.zeros(E * 512, dtype=torch.float32, device=dev)
    net.forward(x, out, E)
    nb.check(nb.lib().nekb_net_raise_copy_timeout())
    with pytest.raises(nb.NekbError, match="did not complete in time") as ei:
        net.forward(x, out, E)
    assert ei.value.code == nb.ERR_CUDA
    net.forward(x, out, E)  # the flag was cleared with the report
    bp = nb.BP(7, 3, 3, 3, perturb=0.1, seed=3)
    L = bp.Nlocal
    lam = torch.cat([torch.full((L,), 1.0), torch.full((L,), 1.5)]).double().to(dev)
    f = torch.from_numpy(O.uniform(L, 8, 3, -1, 1)).to(dev)
    bp.ogs.gather_scatter_many(f)
    nb.check(nb.lib().nekb_net_raise_copy_timeout())
    with pytest.raises(nb.NekbError, match="did not complete in time"):
        bp.pcg(lam, f.clone(), torch.zeros_like(f), 1e-8, 2000, solver=nb.SOLVER_MIXED,
               precond=nb.PRECOND_LEARNED, net=net)
    st = bp.pcg(lam, f.clone(), torch.zeros_like(f), 1e-8, 2000, solver=nb.SOLVER_MIXED,
                precond=nb.PRECOND_LEARNED, net=net)
    assert st["status"] == 0 and st["true_rel_res"] <= 1e-8
