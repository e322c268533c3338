"""nekBone driver on the GB300 library: one benchmark problem, a correctness
check and timed solves, with the reference's summary (nekBone/main.cpp:35-230).

  python -m nekbench_gb300.nekbone [--bp-mode] [--nx 16 --ny 16 --nz 32] [--N 7]
      [--nfields 1] [--solver fp64|fp64_split|mixed] [--inner fp32|bf16|fp32_trilinear]
      [--precond jacobi|copy|learned] [--tol 1e-8] [--maxit 1000] [--fixed]
      [--repetitions 1]

--bp-mode is the reference's BPMODE (nekBone/setup.cpp:44-53): periodic
unperturbed box [-1,1]^3, Poisson (BK), COPY preconditioner, zero-mean rhs and
solution, rhs 3 pi^2 JW cos(pi x) cos(pi y) cos(pi z) assembled by
gather-scatter (setup.cpp:76-98); the correctness check compares with
cos(pi x) cos(pi y) cos(pi z) (main.cpp:105-131).  Without it: the perturbed
unit box with homogeneous Dirichlet boundaries, lambda0 = 1, lambda1 = 1.1
(setup.cpp:51) and a seeded U[-1,1] assembled rhs.  Throughput, bandwidth and
flop figures use the reference's formulas (main.cpp:156-177).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

WORD = 8  # the reference's dfloat = double


def parse(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--bp-mode", action="store_true")
    p.add_argument("--nx", type=int, default=16)
    p.add_argument("--ny", type=int, default=16)
    p.add_argument("--nz", type=int, default=32)
    p.add_argument("--N", type=int, default=7)
    p.add_argument("--nfields", type=int, default=1, choices=(1, 3))
    p.add_argument("--solver", default="fp64", choices=("fp64", "fp64_split", "mixed"))
    p.add_argument("--inner", default="fp32", choices=("fp32", "bf16", "fp32_trilinear"))
    p.add_argument("--precond", default=None, choices=("jacobi", "copy", "learned"))
    p.add_argument("--weights", default=os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                      "weights", "precond_n7_c16.bin"))
    p.add_argument("--inference", default="tensor", choices=("tensor", "tc5", "sync", "fp32"),
                   help="network arithmetic: the default tensor-core kernel, tcgen05, mma.sync "
                        "or FP32 cores")
    p.add_argument("--tol", type=float, default=1e-8)
    p.add_argument("--maxit", type=int, default=1000)
    p.add_argument("--fixed", action="store_true", help="FIXED ITERATION COUNT: exactly maxit")
    p.add_argument("--repetitions", type=int, default=1)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--json", action="store_true", help="print one JSON line instead of text")
    return p.parse_args(argv)


def throughput(it, N, Nq, E, nfields, bk, elapsed):
    """GDOF/s per iteration, GB/s and GFLOP/s as nekBone reports them
    (nekBone/main.cpp:156-177)."""
    Nlocal = Nq ** 3 * E
    gdofs = nfields * it * (N ** 3 * E) / elapsed / 1e9
    gb_ax = (7 + 2 * nfields) * Nlocal + (2 * nfields * Nlocal if bk else 0)
    gbytes = (nfields * Nlocal + 2 * nfields * Nlocal + gb_ax + 3 * (2 * nfields + 1) * Nlocal
              + 4 * nfields * Nlocal) * WORD / 1e9
    fl_ax = nfields * Nlocal * (12 * Nq + 15) + (0 if bk else 5 * nfields * Nlocal)
    flops = 2 * nfields * Nlocal + fl_ax + 3 * 3 * nfields * Nlocal + 4 * nfields * Nlocal
    return gdofs, it * gbytes / elapsed, it * flops / elapsed / 1e9


def main(argv=None):
    a = parse(argv)
    import torch

    import nekbench_gb300 as nb
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    precond = a.precond or ("copy" if a.bp_mode else "jacobi")
    if a.bp_mode:
        bp = nb.BP(a.N, a.nx, a.ny, a.nz, Nfields=a.nfields, periodic=True, dirichlet=False,
                   perturb=0.0, box=(-1.0, 1.0), seed=a.seed)
    else:
        bp = nb.BP(a.N, a.nx, a.ny, a.nz, Nfields=a.nfields, perturb=0.1, seed=a.seed)
    L, E, Np = bp.Nlocal, bp.E, bp.Np
    lam = torch.empty(2 * L, dtype=torch.float64, device=dev)
    lam[:L] = 1.0
    lam[L:] = 0.0 if a.bp_mode else 1.1
    exact = None
    if a.bp_mode:
        X, Y, Z = (bp.device_array(c, L, torch.float64) for c in "xyz")
        JW = bp.device_array("ggeo", 7 * L, torch.float64).view(E, 7, Np)[:, 0, :].reshape(-1)
        exact = torch.cos(math.pi * X) * torch.cos(math.pi * Y) * torch.cos(math.pi * Z)
        f1 = (3 * math.pi ** 2) * JW * exact
        f = f1.repeat(a.nfields)
    else:
        f = torch.empty(a.nfields * L, dtype=torch.float64, device=dev)
        nb.fill_uniform(f, a.seed, 3, -1.0, 1.0)
    bp.ogs.gather_scatter_many(f, k=a.nfields, stride=L)
    kw = dict(solver={"fp64": nb.SOLVER_FP64, "fp64_split": nb.SOLVER_FP64_SPLIT,
                      "mixed": nb.SOLVER_MIXED}[a.solver],
              precond={"jacobi": nb.PRECOND_JACOBI, "copy": nb.PRECOND_COPY,
                       "learned": nb.PRECOND_LEARNED}[precond],
              bk=a.bp_mode, zero_mean=a.bp_mode,
              inner_precision={"fp32": nb.FP32, "bf16": nb.BF16,
                               "fp32_trilinear": nb.FP32_TRILINEAR}[a.inner])
    if precond == "learned":
        kw["net"] = nb.Net.load(a.weights)
        kw["net"].inference = {"tensor": nb.NET_TENSOR, "tc5": nb.NET_TENSOR_TC5,
                               "sync": nb.NET_TENSOR_SYNC, "fp32": nb.NET_FP32}[a.inference]
        kw["solver"] = nb.SOLVER_MIXED
    lam_arg = None if a.bp_mode else lam

    # correctness check / warm-up solve (main.cpp:100-131)
    r, x = f.clone(), torch.zeros_like(f)
    st = bp.pcg(lam_arg, r, x, a.tol if a.tol > 0 else 1e-8, a.maxit, **kw)
    check = {"iterations": st["iterations"], "true_rel_res": st["true_rel_res"]}
    if exact is not None:
        check["max_error"] = float((x.view(a.nfields, L) - exact).abs().max())

    elapsed = 0.0
    for _ in range(a.repetitions):
        r.copy_(f)
        x.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = bp.pcg(lam_arg, r, x, 0.0 if a.fixed else a.tol, a.maxit,
                    fixed_iterations=a.fixed, **kw)
        torch.cuda.synchronize()
        elapsed += time.perf_counter() - t0
    elapsed /= a.repetitions
    it = st["iterations"]
    gdofs, gbs, gflops = throughput(it, a.N, a.N + 1, E, a.nfields, a.bp_mode, elapsed)
    out = {"polyN": a.N, "Nelements": E, "Nfields": a.nfields, "solver": a.solver,
           "inner": a.inner if a.solver == "mixed" or precond == "learned" else None,
           "precond": precond, "bp_mode": a.bp_mode, "check": check, "iterations": it,
           "status": st["status"], "true_rel_res": st["true_rel_res"],
           "repetitions": a.repetitions, "elapsed_s": elapsed,
           "gdofs_per_iter": gdofs, "bandwidth_gbs": gbs, "gflops": gflops}
    if a.json:
        print(json.dumps(out))
    else:
        if exact is not None:
            print(f"correctness check: maxError = {check['max_error']:g} in "
                  f"{check['iterations']} iterations")
        print("summary")
        print(f"  polyN        : {a.N}")
        print(f"  Nelements    : {E}")
        print(f"  Nfields      : {a.nfields}")
        print(f"  solver       : {a.solver} / {precond}")
        print(f"  iterations   : {it}")
        print(f"  Nrepetitions : {a.repetitions}")
        print(f"  elapsed time : {elapsed:g} s")
        print(f"  throughput   : {gdofs:g} GDOF/s/iter")
        print(f"  bandwidth    : {gbs:g} GB/s")
        print(f"  GFLOPS/s     : {gflops:g}")
    bp.free()
    return out


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    main()
