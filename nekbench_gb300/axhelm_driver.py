"""axhelm benchmark driver on the GB300 library, after the reference's
axhelm/main.cpp: one kernel variant and order on random inputs, timed over
repetitions, reported as GDOF/s, GB/s and GFLOP/s with the reference's
formulas (axhelm/main.cpp:161-169), the bytes counted in the storage type of
the precision (8-byte words for FP64 and double-float, 4 for FP32, 4-byte
fields with 2-byte geometry and lambda for BF16 storage).

  python -m nekbench_gb300.axhelm_driver [--N 7] [--E 262144] [--ndim 1] [--bk]
      [--precision fp64|fp64_split|fp32|bf16] [--steps 100] [--json]

Inputs as the reference driver builds them (axhelm/main.cpp:70-128): Gauss
nodes for D (meshJacobiGQ), uniform random ggeo and q, lambda0 = 1 and
lambda1 = 1.1 (0 in BK mode); here the random numbers are seeded.  The
reference checks its kernel against axhelmReference on the CPU; this driver
reports, for the reduced and double-float precisions, the max-norm difference
to the native FP64 kernel on the same inputs.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

WORD = 8


def parse(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--N", type=int, default=7)
    p.add_argument("--E", type=int, default=262144)
    p.add_argument("--ndim", type=int, default=1, choices=(1, 3))
    p.add_argument("--bk", action="store_true")
    p.add_argument("--precision", default="fp64", choices=("fp64", "fp64_split", "fp32", "bf16"))
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--json", action="store_true")
    return p.parse_args(argv)


def figures(N, E, ndim, bk, seconds, word_field=WORD, word_geom=WORD):
    """GDOF/s, GB/s, GFLOP/s of one application (axhelm/main.cpp:161-169)."""
    Nq = N + 1
    Np = Nq ** 3
    gdofs = ndim * N ** 3 * E / seconds / 1e9
    bytes_el = ndim * 2 * Np * word_field + (7 * Np + (0 if bk else 2 * Np)) * word_geom
    flops_el = ndim * (Np * 12 * Nq + 15 * Np + (0 if bk else 5 * Np))
    return gdofs, bytes_el * E / seconds / 1e9, flops_el * E / seconds / 1e9


def main(argv=None):
    a = parse(argv)
    import numpy as np
    import torch

    import nekbench_gb300 as nb
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    N, E, nd = a.N, a.E, a.ndim
    Nq = N + 1
    Np = Nq ** 3
    L = E * Np
    r = np.zeros(Nq)
    w = np.zeros(Nq)
    nb.check(nb.lib().nekb_gauss(N, r.ctypes.data, w.ctypes.data))
    Dh = np.zeros(Nq * Nq)
    nb.check(nb.lib().nekb_dmatrix(Nq, r.ctypes.data, Dh.ctypes.data))
    D64 = torch.from_numpy(Dh).to(dev)
    ggeo = torch.empty(7 * L, dtype=torch.float64, device=dev)
    nb.fill_uniform(ggeo, a.seed, 1, 0.0, 1.0)
    q = torch.empty(nd * L, dtype=torch.float64, device=dev)
    nb.fill_uniform(q, a.seed, 2, 0.0, 1.0)
    lam = torch.empty(2 * L, dtype=torch.float64, device=dev)
    lam[:L] = 1.0
    lam[L:] = 0.0 if a.bk else 1.1
    flags = (nb.AX_BK if a.bk else 0) | (nb.AX_N3 if nd == 3 else 0)
    prec = {"fp64": nb.FP64, "fp64_split": nb.FP64_SPLIT, "fp32": nb.FP32, "bf16": nb.BF16}[a.precision]
    if prec in (nb.FP64, nb.FP64_SPLIT):
        gg, DD, la, qq = ggeo, D64, lam, q
        out = torch.empty_like(q)
    else:
        st = torch.bfloat16 if prec == nb.BF16 else torch.float32
        gg, DD, la = ggeo.to(st), D64.float(), lam.to(st)
        qq = q.float()
        out = torch.empty_like(qq)
    la_arg = None if a.bk else la
    nb.axhelm(Nq, flags, prec, E, L, gg, DD, la_arg, qq, out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.steps):
        nb.axhelm(Nq, flags, prec, E, L, gg, DD, la_arg, qq, out)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) * 1e-3 / a.steps
    wf, wg = {nb.FP64: (8, 8), nb.FP64_SPLIT: (8, 8), nb.FP32: (4, 4), nb.BF16: (4, 2)}[prec]
    gdofs, gbs, gflops = figures(N, E, nd, a.bk, sec, wf, wg)
    res = {"N": N, "Nelements": E, "Ndim": nd, "bk": a.bk, "precision": a.precision,
           "repetitions": a.steps, "ms": sec * 1e3, "gdofs": gdofs, "gbs": gbs, "gflops": gflops}
    if prec != nb.FP64:
        ref = torch.empty_like(q)
        nb.axhelm(Nq, flags, nb.FP64, E, L, ggeo, D64, None if a.bk else lam, q, ref)
        torch.cuda.synchronize()
        res["max_diff_to_fp64"] = float((out.double() - ref).abs().max())
        res["max_rel_diff_to_fp64"] = res["max_diff_to_fp64"] / float(ref.abs().max())
    if a.json:
        print(json.dumps(res))
    else:
        print(f"N={N} Ndim={nd} Nelements={E} {a.precision}{' BK' if a.bk else ''}: "
              f"{sec * 1e3:.3f} ms, {gdofs:.3f} GDOF/s, {gbs:.1f} GB/s, {gflops:.1f} GFLOP/s"
              + (f", max diff to FP64 {res['max_diff_to_fp64']:.3e}" if "max_diff_to_fp64" in res else ""))
    return res


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    main()
