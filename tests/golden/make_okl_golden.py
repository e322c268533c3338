"""Generates tests/golden/okl_serial.npz: outputs of the reference's OKL
kernels, compiled with OCCA's Serial-mode semantics by oracle/okl_serial.py,
on seeded inputs.

Kernels (reference file:line):
  gatherScatterMany_doubleAdd  3rdParty/ogs/okl/gatherScatterMany.okl:58
  updateJacobi                 nekBone/kernel/updateJacobi.okl:27
  weightedInnerProductUpdate   nekBone/kernel/utils.okl:687
  BPUpdatePCG                  nekBone/kernel/utils.okl:795
  weightedInnerProduct2_v0     dot/kernel/VOLTA/dot.okl:27
  weightedBlockInnerProduct2   dot/kernel/VOLTA/dot.okl:67
  advCubatureHex3D_v0          adv/kernel/VOLTA/adv.okl:27 (cubNq = Nq)

Inputs are rebuilt by the tests from the same seeds (the oracle's counter-based
generator and box mesh); the fixture keeps the outputs and a few input samples
that confirm the rebuild.  Run where the nekBench sources are available:

  python oracle/okl_serial.py --tree <nekBench tree>
  python tests/golden/make_okl_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import oracle as O  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def _lib(tag):
    path = os.path.join(REF, f"libokl_{tag}.so")
    if not os.path.exists(path):
        raise SystemExit(f"{path} missing: run python oracle/okl_serial.py --tree <nekBench tree>")
    return C.CDLL(path)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


# ------------------------------------------------------------------ inputs (shared with the tests)
def gs_inputs(signed):
    m = O.BoxMesh(3, 3, 2, 2)
    ids = m.ids.copy()
    if signed:
        flip = O.uniform(m.Nlocal, 41, 0) < 0.5
        ids[flip] *= -1
    return m, ids


def jacobi_inputs(Nq):
    m = O.BoxMesh(Nq - 1, 3, 2, 2, perturb=0.1, seed=40 + Nq)
    L = m.Nlocal
    lam = np.concatenate([O.uniform(L, 42, 1, 0.5, 1.5), O.uniform(L, 42, 2, 0.5, 2.0)])
    mapB = np.zeros(L, np.int32)
    mapB[m.maskIds] = 1
    return m, lam, mapB


def dot_inputs(N):
    return [O.uniform(N, 43, s, 0.0, 1.0) for s in range(3)]


def adv_inputs(Nq, E=3):
    Np = Nq ** 3
    return (O.uniform(12 * E * Np, 44, 0, 0, 1), O.uniform(12 * E * Np, 44, 1, 0, 1),
            O.uniform(Nq * Nq, 44, 2, -1, 1), O.uniform(Nq * Nq, 44, 3, 0, 1),
            O.uniform(3 * E * Np, 44, 4, -1, 1))


def utils_inputs(N, nf):
    off = N + 7
    return (off, O.uniform(N, 45, 0, 0, 1), O.uniform(nf * off, 45, 1, -1, 1),
            O.uniform(nf * off, 45, 2, -1, 1))


GS_FIELDS = (1, 3)
JACOBI_NQ = (4, 8)
DOT_CASES = ((256, 1), (256, 255), (256, 1000), (256, 100003), (512, 100003), (1024, 100003))
ADV_NQ = (4, 8)
UTILS_N = 5003
ALPHA = 0.37


def main(path=None):
    out = {}
    gsl = _lib("gs")
    for signed in (False, True):
        m, ids = gs_inputs(signed)
        Ng, offs, gids, _ = O.ogs_setup(ids)
        for k in GS_FIELDS:
            stride = m.Nlocal + 5
            q = O.uniform(k * stride, 46, k, -1, 1)
            gsl.gatherScatterMany_doubleAdd(C.c_int(Ng), C.c_int(k), C.c_int(stride), _p(offs),
                                            _p(gids), _p(q))
            out[f"gs_s{int(signed)}_k{k}"] = q
    for nq in JACOBI_NQ:
        m, lam, mapB = jacobi_inputs(nq)
        diag = np.zeros(m.Nlocal)
        _lib(f"jacobi_nq{nq}").updateJacobi(C.c_int(m.E), C.c_int(m.Nlocal), _p(mapB), _p(m.ggeo),
                                            _p(m.D), _p(lam), _p(diag))
        out[f"jacobi_nq{nq}"] = diag
        out[f"jacobi_nq{nq}_ggeo_samples"] = m.ggeo[::97].copy()
    for bs, N in DOT_CASES:
        dl = _lib(f"dot_bs{bs}")
        w, x, y = dot_inputs(N)
        nb = (N + bs - 1) // bs
        p0, pb = np.zeros(nb), np.zeros(nb)
        dl.weightedInnerProduct2_v0(C.c_int(N), _p(w), _p(x), _p(y), _p(p0))
        dl.weightedBlockInnerProduct2(C.c_int(N), C.c_int(N), _p(w), _p(x), _p(y), _p(pb))
        out[f"dot_v0_bs{bs}_n{N}"] = p0
        out[f"dot_block_bs{bs}_n{N}"] = pb
    for nq in ADV_NQ:
        vgeo, cub, cubD, It, U = adv_inputs(nq)
        E = 3
        NU = np.zeros(3 * E * nq ** 3)
        _lib(f"adv_nq{nq}").advCubatureHex3D_v0(C.c_int(E), _p(vgeo), _p(cub), _p(cubD), _p(It),
                                                C.c_int(E * nq ** 3), _p(U), _p(NU))
        out[f"adv_nq{nq}"] = NU
    for nf in (1, 3):
        ul = _lib(f"utils_nf{nf}")
        off, w, x, y = utils_inputs(UTILS_N, nf)
        nb = (UTILS_N + 255) // 256
        wxy = np.zeros(2 * nb)
        ul.weightedInnerProductUpdate(C.c_int(UTILS_N), C.c_int(off), C.c_int(nb), _p(w), _p(x),
                                      _p(y), _p(wxy))
        out[f"wip_nf{nf}"] = wxy
        xx, rr = x[:UTILS_N].copy(), y[:UTILS_N].copy()
        ul.BPUpdatePCG(C.c_int(UTILS_N), C.c_double(ALPHA), _p(w), _p(y[:UTILS_N].copy()), _p(xx),
                       _p(rr))
        out[f"update_nf{nf}_x"], out[f"update_nf{nf}_r"] = xx, rr
    out["uniform_check"] = O.uniform(8, 43, 0, 0.0, 1.0)
    path = path or os.path.join(HERE, "okl_serial.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")
    return path


if __name__ == "__main__":
    main()
