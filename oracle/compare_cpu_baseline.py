"""Times the CPU baseline (cpu_axhelm.c) against the reference's own CPU
axhelm (axhelm/kernel/CPU/axhelm.c compiled unmodified with the reference's
flags: make -C oracle ref-fast REF=<nekBench tree>) on the same inputs, the
same elements and the same OpenMP threads, and checks that both agree with the
bit-identical checker.  FP64 axhelm_bk_v0 and axhelm_v0, N=7 by default.

  python oracle/compare_cpu_baseline.py [--N 7] [--n 16] [--reps 20]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import oracle as O  # noqa: E402


def median_rate(fn, E, N, reps):
    fn()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return E * N ** 3 / float(np.median(ts)) / 1e9


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--N", type=int, default=7)
    ap.add_argument("--n", type=int, default=16)
    ap.add_argument("--reps", type=int, default=20)
    a = ap.parse_args()
    N, Nq = a.N, a.N + 1
    R = O.ref(Nq, fast=True)
    if R is None:
        sys.exit("oracle/_ref/libnekref_fast_nq%d.so missing: make -C oracle ref-fast REF=..." % Nq)
    m = O.BoxMesh(N, a.n, a.n, a.n, perturb=0.1, seed=1)
    E, L = m.E, m.Nlocal
    q = O.uniform(L, 1, 3, -1, 1)
    lam = np.concatenate([O.uniform(L, 1, 1, 0.5, 1.5), O.uniform(L, 1, 2, 0.5, 2.0)])
    out = {"N": N, "E": E, "threads": O.omp_threads()}
    for name, bk in (("bk", 1), ("helmholtz", 0)):
        la = np.concatenate([np.ones(L), np.zeros(L)]) if bk else lam
        A_ref, A_port = np.zeros(L), np.zeros(L)
        ref_rate = median_rate(lambda: R.nekref_axhelm_cpu(bk, E, L, m.ggeo, m.D, la.ctypes.data,
                                                           q, A_ref), E, N, a.reps)
        port_rate = median_rate(lambda: O.cpu_axhelm(Nq, bk, E, L, m.ggeo, m.D, la, q, A_port),
                                E, N, a.reps)
        check = O.axhelm(Nq, E, L, O.AX_BK if bk else 0, m.ggeo, m.D, la, q)
        scale = np.abs(check).max()
        out[name] = {"reference_gdofs": ref_rate, "port_gdofs": port_rate,
                     "port_over_reference": port_rate / ref_rate,
                     "port_vs_checker": float(np.abs(A_port - check).max() / scale),
                     "reference_vs_checker": float(np.abs(A_ref - check).max() / scale)}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
