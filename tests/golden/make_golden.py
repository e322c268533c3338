"""Generates the golden vectors under tests/golden/ from the reference itself.

Run in a checkout where the nekBench sources are available and oracle/_ref was
built (``make -C oracle ref``): the outputs come from the reference's own
axhelm/axhelmReference.cpp, axhelm/kernel/CPU/axhelm.c and
nekBone/kernel/CPU/weightedInnerProduct.c, compiled unmodified.  Inputs are
seeded (the oracle's counter-based generator and box mesh), so the fixtures
are reproducible:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle as O  # noqa: E402


def axhelm_case(N, nx, ny, nz, seed):
    Nq = N + 1
    R = O.ref(Nq)
    assert R is not None, f"oracle/_ref/libnekref_nq{Nq}.so missing: run make -C oracle ref"
    m = O.BoxMesh(N, nx, ny, nz, perturb=0.1, seed=seed)
    E, L = m.E, m.Nlocal
    lam = np.concatenate([O.uniform(L, seed, 1, 0.5, 1.5), O.uniform(L, seed, 2, 0.5, 2.0)])
    q = O.uniform(3 * L, seed, 3, -1.0, 1.0)
    out = {"N": N, "E": E, "ggeo": m.ggeo, "D": m.D, "lam": lam, "q": q}
    for variant in range(4):  # bit0 BK, bit1 n3
        nf = 3 if variant & 2 else 1
        Aq = np.zeros(nf * L)
        R.nekref_axhelm_cpu(variant, E, L, m.ggeo, m.D, lam.ctypes.data, q[: nf * L].copy(), Aq)
        out[f"Aq_cpu_v{variant}"] = Aq
    for lam1 in (0.0, 1.1):
        Aq = np.zeros(L)
        R.nekref_axhelm_reference(Nq, E, lam1, m.ggeo, m.D, q[:L].copy(), Aq)
        out[f"Aq_reference_lam{lam1}"] = Aq
    return out


def config1_case(seed=1, stride=61):
    """axhelm FP64 Poisson at N=7 on the perturbed 8x8x8 box (E=512, 262,144
    local nodes): axhelmReference.cpp with lambda=0 (the BK operator).  The
    full output is 2 MB, so the fixture keeps every stride-th node and the
    whole array's sum, sum of squares and max-abs; the inputs are rebuilt from
    the seed by the oracle's box mesh and generator."""
    N, n = 7, 8
    Nq = N + 1
    R = O.ref(Nq)
    assert R is not None, f"oracle/_ref/libnekref_nq{Nq}.so missing: run make -C oracle ref"
    m = O.BoxMesh(N, n, n, n, perturb=0.1, seed=seed)
    E, L = m.E, m.Nlocal
    q = O.uniform(L, seed, 3, -1.0, 1.0)
    Aq = np.zeros(L)
    R.nekref_axhelm_reference(Nq, E, 0.0, m.ggeo, m.D, q.copy(), Aq)
    idx = np.arange(0, L, stride, dtype=np.int64)
    return {"N": N, "n": n, "seed": seed, "idx": idx, "Aq_samples": Aq[idx],
            "ggeo_samples": m.ggeo[idx], "q_samples": q[idx],
            "Aq_sum": Aq.sum(), "Aq_sumsq": (Aq * Aq).sum(), "Aq_maxabs": np.abs(Aq).max()}


def wip_case(Nq, n, seed):
    R = O.ref(Nq)
    w = O.uniform(n, seed, 1, 0.1, 1.0)
    a = O.uniform(n, seed, 2, -1.0, 1.0)
    b = O.uniform(n, seed, 3, -1.0, 1.0)
    wab = np.zeros(2)
    R.nekref_weighted_inner_product_update(n, n, w, a, b, wab)
    return {"w": w, "a": a, "b": b, "wab": wab}


def main():
    np.savez_compressed(os.path.join(HERE, "axhelm_n3.npz"), **axhelm_case(3, 2, 2, 2, 11))
    np.savez_compressed(os.path.join(HERE, "axhelm_n7.npz"), **axhelm_case(7, 2, 1, 1, 12))
    np.savez_compressed(os.path.join(HERE, "axhelm_n9.npz"), **axhelm_case(9, 1, 1, 1, 13))
    np.savez_compressed(os.path.join(HERE, "weighted_inner_product.npz"), **wip_case(8, 1000, 14))
    np.savez_compressed(os.path.join(HERE, "axhelm_config1_e512.npz"), **config1_case())
    rng = {"u_seed5_stream2": O.uniform(16, 5, 2), "u_seed0_stream0": O.uniform(16, 0, 0)}
    np.savez_compressed(os.path.join(HERE, "uniform.npz"), **rng)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
