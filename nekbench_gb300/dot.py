"""dot benchmark driver on the GB300 library, after the reference's dot/main.cpp:
the weighted inner product of three node arrays of N^3-order elements, as
per-block partials on the GPU that the host sums in block order
(weightedInnerProduct, dot/main.cpp:27-48), timed over repetitions and reported
with the reference's formulas (dot/main.cpp:157-159): GDOF/s = Nelements N^3 /
time, GB/s = 3 Np 8 Nelements / time.

  python -m nekbench_gb300.dot [--N 7] [--E 262144] [--block 256]
      [--kernel weightedInnerProduct2_v0|weightedInnerProduct2_v1|weightedBlockInnerProduct2]
      [--steps 100] [--json]

The reference fills the three arrays with drand48 (and, as written, uploads
the same array three times, dot/main.cpp:129-135); here they are three seeded
uniform arrays.  Two times are reported: the reference's (kernel + copy of
the partials to the host + the host sum, per call) and the kernel's alone
(CUDA events).
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np


def parse(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--N", type=int, default=7)
    p.add_argument("--E", type=int, default=262144)
    p.add_argument("--block", type=int, default=256)
    p.add_argument("--kernel", default="weightedInnerProduct2_v0")
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--json", action="store_true")
    return p.parse_args(argv)


def figures(N, E, seconds):
    """GDOF/s and GB/s as dot/main.cpp:157-159 computes them."""
    Np = (N + 1) ** 3
    return E * N ** 3 / seconds / 1e9, 3 * Np * 8 * E / seconds / 1e9


def main(argv=None):
    a = parse(argv)
    import torch

    import nekbench_gb300 as nb
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    Np = (a.N + 1) ** 3
    L = a.E * Np
    arrs = []
    for s in range(3):
        t = torch.empty(L, dtype=torch.float64, device=dev)
        nb.fill_uniform(t, a.seed, 10 + s, 0.0, 1.0)
        arrs.append(t)
    w, x, y = arrs[2], arrs[0], arrs[1]  # kernel(N, o_c, o_a, o_b, o_tmp), dot/main.cpp:31,146
    kernel = nb.load_dot_kernel(a.kernel, a.block)
    nblock = nb.dot_num_blocks(L, a.block)
    tmp = torch.empty(nblock, dtype=torch.float64, device=dev)
    host = torch.empty(nblock, dtype=torch.float64, pin_memory=True)
    host_np = host.numpy()

    def call():  # weightedInnerProduct (dot/main.cpp:27-48)
        if kernel.variant == nb.DOT_BLOCK:
            kernel(L, L, w, x, y, tmp)
        else:
            kernel(L, w, x, y, tmp)
        host.copy_(tmp)
        return float(np.cumsum(host_np)[-1])  # block order, one addition after another

    wab = call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        wab = call()
    elapsed = (time.perf_counter() - t0) / a.steps
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.steps):
        if kernel.variant == nb.DOT_BLOCK:
            kernel(L, L, w, x, y, tmp)
        else:
            kernel(L, w, x, y, tmp)
    e1.record()
    torch.cuda.synchronize()
    kern = e0.elapsed_time(e1) * 1e-3 / a.steps
    gdofs, gbs = figures(a.N, a.E, elapsed)
    kgdofs, kgbs = figures(a.N, a.E, kern)
    res = {"kernel": a.kernel, "N": a.N, "Nelements": a.E, "blockSize": a.block, "Nblock": nblock,
           "NRepetitions": a.steps, "elapsed_s": elapsed, "gdofs": gdofs, "gbs": gbs,
           "kernel_s": kern, "kernel_gdofs": kgdofs, "kernel_gbs": kgbs, "wab": wab}
    if a.json:
        print(json.dumps(res))
    else:
        print(f"MPItasks=1 NRepetitions={a.steps} N={a.N} Nelements={a.E} blockSize={a.block} "
              f"elapsed time={elapsed:g} GDOF/s={gdofs:g} GB/s={gbs:g} "
              f"(kernel alone {kern:g} s, {kgbs:g} GB/s)")
    return res


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    main()
