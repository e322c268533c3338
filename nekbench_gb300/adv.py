"""adv benchmark driver on the GB300 library, after the reference's adv/main.cpp:
advCubatureHex3D_v0 on random inputs, timed over repetitions, reported as
GDOF/s = Nelements N^3 / time (adv/main.cpp:142).  The reference prints no
bandwidth or flop figure; this driver adds the FP64 flops it counts (`flops`)
and the bytes the operator must move (`bytes`), against which the GPU's FP64
and HBM roofs are read.

  python -m nekbench_gb300.adv [--N 7] [--cubN 11] [--E 8192] [--steps 10]
      [--precision fp64|fp64_split] [--json]

fp64_split evaluates the same operator in double-float arithmetic on the FP32
pipes and reports its max-norm difference to the FP64 kernel on the same
inputs.

Inputs as the reference driver builds them (adv/main.cpp:98-112): uniform
random vgeo, cubvgeo, cubD, cubInterpT and U (here seeded).
"""
from __future__ import annotations

import argparse
import json
import os
import sys


def parse(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--N", type=int, default=7)
    p.add_argument("--cubN", type=int, default=11)
    p.add_argument("--E", type=int, default=8192)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--precision", default="fp64", choices=("fp64", "fp64_split"))
    p.add_argument("--json", action="store_true")
    return p.parse_args(argv)


def flops(Nq, cq):
    """FP64 flops of one element (an FMA counts 2): interpolation and projection
    (3 fields, 3 directions each), 3 cubature derivatives of 3 fields, the
    contravariant velocity and the advection term per cubature node, the
    inverse mass per GLL node."""
    tensor = Nq ** 3 * cq + Nq ** 2 * cq ** 2 + Nq * cq ** 3
    return 2 * 2 * 3 * tensor + 2 * 3 * 3 * cq ** 4 + 33 * cq ** 3 + 3 * Nq ** 3


def bytes_moved(Nq, cq):
    """Bytes one element must move: 10 cubature metric slots, the IJW slot, U
    and NU (3 fields each), 8-byte words."""
    return 8 * (10 * cq ** 3 + Nq ** 3 + 6 * Nq ** 3)


def main(argv=None):
    a = parse(argv)
    import torch

    import nekbench_gb300 as nb
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    Nq, cq, E = a.N + 1, a.cubN + 1, a.E
    Np, cNp = Nq ** 3, cq ** 3

    def rand(n, stream):
        t = torch.empty(n, dtype=torch.float64, device=dev)
        nb.fill_uniform(t, a.seed, stream, 0.0, 1.0)
        return t
    vgeo, cubvgeo = rand(12 * E * Np, 20), rand(12 * E * cNp, 21)
    cubD, cubI = rand(cq * cq, 22), rand(Nq * cq, 23)
    U = rand(3 * E * Np, 24)
    NU = torch.empty_like(U)
    prec = nb.FP64_SPLIT if a.precision == "fp64_split" else nb.FP64
    kernel = nb.load_adv_kernel(a.N, a.cubN, prec)
    kernel(E, vgeo, cubvgeo, cubD, cubI, E * Np, U, NU)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.steps):
        kernel(E, vgeo, cubvgeo, cubD, cubI, E * Np, U, NU)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) * 1e-3 / a.steps
    res = {"N": a.N, "cubN": a.cubN, "Nelements": E, "precision": a.precision,
           "NRepetitions": a.steps, "elapsed_s": sec,
           "gdofs": E * a.N ** 3 / sec / 1e9, "gflops": flops(Nq, cq) * E / sec / 1e9,
           "gbs": bytes_moved(Nq, cq) * E / sec / 1e9,
           "flops_per_element": flops(Nq, cq), "bytes_per_element": bytes_moved(Nq, cq)}
    if prec != nb.FP64:
        ref = torch.empty_like(U)
        nb.load_adv_kernel(a.N, a.cubN)(E, vgeo, cubvgeo, cubD, cubI, E * Np, U, ref)
        torch.cuda.synchronize()
        res["max_rel_diff_to_fp64"] = float((NU - ref).abs().max() / ref.abs().max())
    if a.json:
        print(json.dumps(res))
    else:
        print(f"MPItasks=1 NRepetitions={a.steps} N={a.N} cubN={a.cubN} Nelements={E} "
              f"elapsed time={sec:g} GDOF/s={res['gdofs']:g} "
              f"(FP64 {res['gflops']:.1f} GFLOP/s, {res['gbs']:.1f} GB/s)")
    return res


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    main()
