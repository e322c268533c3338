"""Training and evaluation of the learned element preconditioner.

Data: residuals that the plain Jacobi-PCG itself produces, paired with a
correction.  For each seeded problem (lambda0 = 1, lambda1 = 1 + 0.5
sin(2 pi k.x) with k ~ U{1..4}^3, f ~ U[-1,1] assembled), the FP32 Jacobi-PCG
iterate x_k after k iterations (k spread over the whole solve: SNAPSHOT_FRACTIONS
of its iteration count) gives the residual
r_k = b - A x_k (FP64).  The default correction is the element-local block
solve of r_k (exact on each element's interior nodes, Jacobi on its boundary),
a fixed linear map of the element's own residual that a local network can
represent; the alternative is the correction the same PCG makes over its next
`horizon` iterations, x_{k+horizon} - x_k (horizon=0: the remaining global
error x* - x_k), which depends on the residual outside the element.  A random
subset of elements of each snapshot becomes training pairs through the
library's nekb_net_prepare_pairs (element RMS normalisation, Jacobi part
removed).

Training runs the network's own fused forward/backward kernels and Adam
(nekb_net_train_step); evaluation compares flexible PCG with the network
against Jacobi-PCG to the same true FP64 relative residual.  The network is
nonlinear, so the flexible iteration keeps several directions (FCG(m), m = 5
by default): with the single-direction flexible beta the Krylov space loses
conjugacy over a long solve and the network costs iterations instead of
saving them.  torch only holds
device buffers and gathers element subsets.
"""
from __future__ import annotations

import math
import time

import numpy as np

import nekbench_gb300 as nb

# residual snapshots spread over a whole Jacobi-PCG solve (fractions of its
# iteration count): late residuals are smooth across elements and must be in
# the training set too
SNAPSHOT_FRACTIONS = (0.0, 0.02, 0.08, 0.2, 0.35, 0.5, 0.65, 0.8, 0.95)


def snapshot_schedule(bp, lam, f, torch, dev, fractions=SNAPSHOT_FRACTIONS):
    """Iteration numbers at the given fractions of the Jacobi-PCG iteration
    count (to relative residual 1e-8) of this problem."""
    r = f.clone()
    x = torch.zeros_like(f)
    st = bp.pcg(lam, r, x, 1e-8, 20000, solver=nb.SOLVER_MIXED)
    n = max(int(st["iterations"]), 1)
    return sorted({int(round(q * n)) for q in fractions})


def coefficients(bp, seed, torch):
    L = bp.Nlocal
    x = bp.device_array("x", L, torch.float64)
    y = bp.device_array("y", L, torch.float64)
    z = bp.device_array("z", L, torch.float64)
    k = np.random.default_rng(seed).integers(1, 5, size=3)
    lam = torch.ones(2 * L, dtype=torch.float64, device=x.device)
    lam[L:] = 1.0 + 0.5 * torch.sin(2.0 * math.pi * (k[0] * x + k[1] * y + k[2] * z))
    return lam


def rhs(bp, seed, torch, dev):
    f = torch.empty(bp.Nlocal, dtype=torch.float64, device=dev)
    nb.fill_uniform(f, seed, 3, -1.0, 1.0)
    bp.ogs.gather_scatter_many(f)
    return f


def generate_pairs(bp, seeds, torch, dev, frac=0.125, snapshots=None, horizon=16, log=None,
                   target="local"):
    """Training pairs (inp, target), float32 device tensors of shape [M, Np].

    target="local": the correction paired with the residual r_k is the
    element-local block solve of r_k (element-interior Helmholtz solve, Jacobi
    on the element boundary; nekb_bp_local_correction), a fixed linear map of
    the element's residual.
    target="pcg": x_{k+horizon} - x_k, what the Jacobi-PCG itself adds to its
    iterate over the next `horizon` iterations (horizon=0: the remaining error
    x* - x_k)."""
    if target not in ("local", "pcg"):
        raise ValueError(f"unknown target {target!r}")
    if target == "local":
        horizon = 1  # no reference solve needed
    E, Np, L = bp.E, bp.Np, bp.Nlocal
    n_sel = max(1, int(frac * E))
    r = torch.empty(L, dtype=torch.float64, device=dev)
    x = torch.empty(L, dtype=torch.float64, device=dev)
    xs = torch.empty(L, dtype=torch.float64, device=dev)
    inps, tgts = [], []
    t0 = time.perf_counter()
    for s in seeds:
        lam = coefficients(bp, s, torch)
        f = rhs(bp, s, torch, dev)
        snaps = snapshots if snapshots is not None else snapshot_schedule(bp, lam, f, torch, dev)
        if horizon <= 0:
            r.copy_(f)
            xs.zero_()
            bp.pcg(lam, r, xs, 1e-9, 20000, solver=nb.SOLVER_MIXED)  # converged reference
        inv_diag = None
        rng = np.random.default_rng(10_000 + s)
        for k in snaps:
            if horizon > 0 and target == "pcg":
                r.copy_(f)
                xs.zero_()
                bp.pcg(lam, r, xs, 0.0, k + horizon, solver=nb.SOLVER_MIXED,
                       fixed_iterations=True, max_outer=1)
            r.copy_(f)
            x.zero_()
            bp.pcg(lam, r, x, 0.0, k, solver=nb.SOLVER_MIXED, fixed_iterations=True, max_outer=1)
            if inv_diag is None:  # the Jacobi diagonal of this seed's lambda
                inv_diag = bp.device_array("invDiag", L, torch.float64).float().view(E, Np)
            idx = torch.from_numpy(rng.choice(E, n_sel, replace=False).astype(np.int64)).to(dev)
            rk = r.float().view(E, Np).index_select(0, idx).contiguous()
            dk = inv_diag.index_select(0, idx).contiguous()
            if target == "local":
                ek = torch.empty_like(rk)
                bp.local_correction(lam, idx.to(torch.int32), rk, dk, ek)
            else:
                ek = (xs - x).float().view(E, Np).index_select(0, idx).contiguous()
            inp = torch.empty_like(rk)
            tgt = torch.empty_like(rk)
            nb.prepare_pairs(Np, n_sel, n_sel, rk, ek, dk, inp, tgt)
            inps.append(inp)
            tgts.append(tgt)
    torch.cuda.synchronize()
    if log:
        log(f"generated {len(inps) * n_sel} pairs from {len(seeds)} solves in "
            f"{time.perf_counter() - t0:.1f} s")
    return torch.cat(inps), torch.cat(tgts)


def train(net, inp, tgt, torch, steps=2000, batch=2048, lr=1e-3, seed=0, log=None):
    M = inp.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    losses = []
    perm = torch.randperm(M, generator=g).to(inp.device)
    pos = 0
    bi = torch.empty((batch, inp.shape[1]), dtype=torch.float32, device=inp.device)
    bt = torch.empty_like(bi)
    t0 = time.perf_counter()
    for step in range(steps):
        if pos + batch > M:
            perm = torch.randperm(M, generator=g).to(inp.device)
            pos = 0
        idx = perm[pos:pos + batch]
        pos += batch
        torch.index_select(inp, 0, idx, out=bi)
        torch.index_select(tgt, 0, idx, out=bt)
        # cosine decay of the learning rate
        lr_t = lr * 0.5 * (1 + math.cos(math.pi * step / steps))
        losses.append(net.train_step(bi, bt, batch, max(lr_t, 1e-6)))
        if log and (step % 250 == 0 or step == steps - 1):
            log(f"step {step:5d} loss {losses[-1]:.4e} ({time.perf_counter() - t0:.1f} s)")
    return losses


def evaluate(bp, net, seeds, torch, dev, tol=1e-8, inner_precision=None, solver=None,
             fcg_window=0):
    """Iterations and time to `tol` (true FP64 relative residual) with and without
    the network, on the same problems."""
    inner_precision = nb.FP32 if inner_precision is None else inner_precision
    solver = nb.SOLVER_MIXED if solver is None else solver
    r = torch.empty(bp.Nlocal, dtype=torch.float64, device=dev)
    x = torch.empty_like(r)
    rows = []
    for s in seeds:
        lam = coefficients(bp, s, torch)
        f = rhs(bp, s, torch, dev)
        row = {"seed": int(s)}
        maxit = 20000
        for name, kw in (("jacobi", {}), ("learned", {"precond": nb.PRECOND_LEARNED, "net": net,
                                                      "fcg_window": fcg_window})):
            best = None
            for _ in range(2):
                r.copy_(f)
                x.zero_()
                st = bp.pcg(lam, r, x, tol, maxit, solver=solver,
                            inner_precision=inner_precision, **kw)
                if best is None or st["elapsed_s"] < best["elapsed_s"]:
                    best = st
            row[name] = {k: best[k] for k in ("iterations", "outer_iterations", "status",
                                               "true_rel_res", "elapsed_s")}
            # a network that slows convergence is stopped at 3x the Jacobi count
            maxit = 3 * max(best["iterations"], 1)
        rows.append(row)
    it_j = np.mean([r_["jacobi"]["iterations"] for r_ in rows])
    it_l = np.mean([r_["learned"]["iterations"] for r_ in rows])
    t_j = np.mean([r_["jacobi"]["elapsed_s"] for r_ in rows])
    t_l = np.mean([r_["learned"]["elapsed_s"] for r_ in rows])
    return {"seeds": len(rows), "mean_iterations_jacobi": float(it_j),
            "mean_iterations_learned": float(it_l), "iteration_ratio": float(it_j / it_l),
            "mean_time_jacobi_s": float(t_j), "mean_time_learned_s": float(t_l),
            "time_ratio": float(t_j / t_l),
            "all_converged": all(r_[k]["status"] == 0 and r_[k]["true_rel_res"] <= tol
                                 for r_ in rows for k in ("jacobi", "learned")),
            "rows": rows}
