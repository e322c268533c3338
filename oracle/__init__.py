"""CPU oracle for the nekBench hot path -- test infrastructure only.

ctypes/numpy front end over ``liboracle.so`` (a plain-C restatement of the
reference algorithms, ``nekb_oracle.c``) and, where it was built, over
``_ref/libnekref_nq<Nq>.so`` (the reference's own CPU axhelm sources compiled
unmodified).  Only the tests, the smoke check and the benchmark's CPU-baseline
leg import this package; the library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REFS: dict = {}

AX_BK, AX_N3, AX_PARTIAL = 1, 2, 4

_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_vp = C.c_void_p


def build(ref: bool = False) -> None:
    """Compile liboracle.so and libcpuaxhelm.so (and the reference shims when ``ref``)."""
    subprocess.run(["make", "-s", "-C", _HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", _HERE, "ref"], check=True)


def lib():
    global _LIB
    if _LIB is not None:
        return _LIB
    path = os.path.join(_HERE, "liboracle.so")
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    L.nekbo_hash.restype = C.c_uint64
    L.nekbo_hash.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
    L.nekbo_uniform.restype = C.c_double
    L.nekbo_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
    L.nekbo_fill_uniform.argtypes = [_d, C.c_int64, C.c_uint64, C.c_uint64, C.c_double, C.c_double]
    L.nekbo_gll.argtypes = [C.c_int, _d, _d]
    L.nekbo_gauss.argtypes = [C.c_int, _d, _d]
    L.nekbo_dmatrix.argtypes = [C.c_int, _d, _d]
    L.nekbo_box_vertices.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint64, C.c_int,
                                     C.c_double, C.c_double, _d, _d, _d]
    L.nekbo_zero_mean.argtypes = [C.c_int64, C.c_int, C.c_int64, _d]
    L.nekbo_box_ids.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _i64]
    L.nekbo_box_mask.restype = C.c_int64
    L.nekbo_box_mask.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _vp]
    L.nekbo_physical_nodes.argtypes = [C.c_int, C.c_int64, _d, _d, _d, _d, _d, _d, _d]
    L.nekbo_geometric_factors.argtypes = [C.c_int, C.c_int64, _d, _d, _d, _d, _d, _d]
    L.nekbo_axhelm.argtypes = [C.c_int, C.c_int64, C.c_int64, C.c_int, _vp, _d, _d, _vp, _d, _d]
    L.nekbo_axhelm_omp.argtypes = [C.c_int, C.c_int64, C.c_int64, C.c_int, _d, _d, _vp, _d, _d]
    L.nekbo_omp_threads.restype = C.c_int
    L.nekbo_ogs_setup.restype = C.c_int64
    L.nekbo_ogs_setup.argtypes = [C.c_int64, _i64, _i32, _i32, _d]
    L.nekbo_gs_many_add.argtypes = [C.c_int64, _i32, _i32, C.c_int, C.c_int64, _d]
    L.nekbo_mask.argtypes = [C.c_int64, _i32, _d]
    L.nekbo_update_jacobi.argtypes = [C.c_int, C.c_int64, C.c_int64, _vp, _d, _d, _d, _d]
    L.nekbo_pcg.restype = C.c_int
    L.nekbo_pcg.argtypes = [C.POINTER(NekboBP), _d, _d, C.c_double, C.c_int, C.c_int, C.c_int,
                            C.c_int, _vp]
    L.nekbo_bp_apply.argtypes = [C.POINTER(NekboBP), _d, _d]
    L.nekbo_set_cpu_axhelm.argtypes = [C.c_void_p]
    L.nekbo_pcg_omp.restype = C.c_int
    L.nekbo_pcg_omp.argtypes = [C.POINTER(NekboBP), _d, _d, C.c_double, C.c_int, C.c_int, C.c_int,
                                C.POINTER(C.c_double)]
    L.nekbo_conv3d_forward.argtypes = [C.c_int, C.c_int64, C.c_int, C.c_int, _f, _f, _f]
    L.nekbo_conv3d_backward.argtypes = [C.c_int, C.c_int64, C.c_int, C.c_int, _f, _f, _f, _vp, _f]
    L.nekbo_gelu_forward.argtypes = [C.c_int64, _f, _f]
    L.nekbo_gelu_backward.argtypes = [C.c_int64, _f, _f, _f]
    L.nekbo_dot_partials.restype = C.c_int64
    L.nekbo_dot_partials.argtypes = [C.c_int, C.c_int64, C.c_int, C.c_int64, C.c_int, _d, _d, _d, _d]
    L.nekbo_adv_cubature.argtypes = [C.c_int, C.c_int, C.c_int64, _d, _d, _d, _d, C.c_int64, _d, _d]
    _LIB = L
    return L


class NekboBP(C.Structure):
    _fields_ = [
        ("Nq", C.c_int), ("Nelements", C.c_int64), ("Nfields", C.c_int), ("offset", C.c_int64),
        ("bk", C.c_int), ("ggeo", _vp), ("D", _vp), ("lambda_", _vp), ("Ngather", C.c_int64),
        ("gatherOffsets", _vp), ("gatherIds", _vp), ("invDegree", _vp), ("Nmasked", C.c_int64),
        ("maskIds", _vp),
    ]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ----------------------------------------------------------------------------- random numbers
def uniform(n: int, seed: int, stream: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
    v = np.empty(int(n), dtype=np.float64)
    lib().nekbo_fill_uniform(v, int(n), seed, stream, lo, hi)
    return v


# ----------------------------------------------------------------------------- basis
def gll(N: int):
    x = np.zeros(N + 1)
    w = np.zeros(N + 1)
    lib().nekbo_gll(N, x, w)
    return x, w


def gauss(N: int):
    x = np.zeros(N + 1)
    w = np.zeros(N + 1)
    lib().nekbo_gauss(N, x, w)
    return x, w


def dmatrix(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    D = np.zeros(len(x) * len(x))
    lib().nekbo_dmatrix(len(x), x, D)
    return D


# ----------------------------------------------------------------------------- mesh
class BoxMesh:
    """Structured box of nx*ny*nz hexes of order N (oracle construction)."""

    def __init__(self, N, nx, ny, nz, perturb=0.1, seed=1, periodic=False, dirichlet=True,
                 box=(0.0, 0.0)):
        L = lib()
        self.N, self.Nq = N, N + 1
        self.Np = self.Nq ** 3
        self.nx, self.ny, self.nz = nx, ny, nz
        self.E = nx * ny * nz
        self.r, self.w = gll(N)
        self.D = dmatrix(self.r)
        E8 = self.E * 8
        self.EX, self.EY, self.EZ = np.zeros(E8), np.zeros(E8), np.zeros(E8)
        L.nekbo_box_vertices(nx, ny, nz, perturb, seed, int(periodic), float(box[0]), float(box[1]),
                             self.EX, self.EY, self.EZ)
        Nl = self.E * self.Np
        self.ids = np.zeros(Nl, dtype=np.int64)
        L.nekbo_box_ids(N, nx, ny, nz, int(periodic), int(dirichlet), self.ids)
        if dirichlet and not periodic:
            nm = L.nekbo_box_mask(N, nx, ny, nz, None)
            self.maskIds = np.zeros(nm, dtype=np.int32)
            L.nekbo_box_mask(N, nx, ny, nz, _ptr(self.maskIds))
        else:
            self.maskIds = np.zeros(0, dtype=np.int32)
        self.x, self.y, self.z = np.zeros(Nl), np.zeros(Nl), np.zeros(Nl)
        L.nekbo_physical_nodes(N, self.E, self.r, self.EX, self.EY, self.EZ, self.x, self.y, self.z)
        self.ggeo = np.zeros(7 * Nl)
        L.nekbo_geometric_factors(N, self.E, self.w, self.D, self.x, self.y, self.z, self.ggeo)

    @property
    def Nlocal(self):
        return self.E * self.Np


# ----------------------------------------------------------------------------- axhelm
def axhelm(Nq, E, offset, flags, ggeo, D, lam, q, element_list=None, out=None):
    nf = 3 if flags & AX_N3 else 1
    Aq = np.zeros(nf * offset) if out is None else out
    el = None
    if flags & AX_PARTIAL:
        el = np.ascontiguousarray(element_list, dtype=np.int32)
    lam_c = None if lam is None else np.ascontiguousarray(lam, dtype=np.float64)
    lib().nekbo_axhelm(Nq, E, offset, flags, _ptr(el), ggeo, D, _ptr(lam_c), q, Aq)
    return Aq


def axhelm_omp(Nq, E, offset, flags, ggeo, D, lam, q, out):
    lam_c = None if lam is None else np.ascontiguousarray(lam, dtype=np.float64)
    lib().nekbo_axhelm_omp(Nq, E, offset, flags, ggeo, D, _ptr(lam_c), q, out)
    return out


def omp_threads() -> int:
    return lib().nekbo_omp_threads()


# ----------------------------------------------------------------------------- ogs
def ogs_setup(ids: np.ndarray):
    ids = np.ascontiguousarray(ids, dtype=np.int64)
    N = len(ids)
    offsets = np.zeros(N + 1, dtype=np.int32)
    gids = np.zeros(max(N, 1), dtype=np.int32)
    invdeg = np.zeros(max(N, 1))
    Ng = lib().nekbo_ogs_setup(N, ids, offsets, gids, invdeg)
    nl = int(offsets[Ng])
    return int(Ng), offsets[: Ng + 1].copy(), gids[:nl].copy(), invdeg[:N].copy()


def gs_many_add(Ng, offsets, gids, q, k=1, stride=0):
    lib().nekbo_gs_many_add(Ng, offsets, gids, k, stride, q)
    return q


def update_jacobi(Nq, E, offset, ggeo, D, lam, mapB=None):
    diag = np.zeros(E * Nq ** 3)
    mb = None if mapB is None else np.ascontiguousarray(mapB, dtype=np.int32)
    lib().nekbo_update_jacobi(Nq, E, offset, _ptr(mb), ggeo, D, lam, diag)
    return diag


# ----------------------------------------------------------------------------- PCG
class BP:
    """Host copy of a benchmark problem for the oracle PCG."""

    def __init__(self, mesh: BoxMesh, lam: np.ndarray, bk: bool = False, Nfields: int = 1):
        self.mesh = mesh
        self.lam = np.ascontiguousarray(lam, dtype=np.float64)
        self.Ng, self.offs, self.gids, self.invdeg = ogs_setup(mesh.ids)
        self.bk = bk
        self.Nfields = Nfields
        self.s = NekboBP(mesh.Nq, mesh.E, Nfields, mesh.Nlocal, int(bk), _ptr(mesh.ggeo),
                         _ptr(mesh.D), _ptr(self.lam), self.Ng, _ptr(self.offs), _ptr(self.gids),
                         _ptr(self.invdeg), len(mesh.maskIds), _ptr(mesh.maskIds))

    def apply(self, q):
        Aq = np.zeros_like(q)
        lib().nekbo_bp_apply(C.byref(self.s), q, Aq)
        return Aq

    def pcg(self, r, x, tol, maxit, precond=1, flexible=False, fixed=False, hist=False):
        h = np.zeros(maxit + 1) if hist else None
        it = lib().nekbo_pcg(C.byref(self.s), r, x, tol, maxit, precond, int(flexible), int(fixed),
                             _ptr(h))
        return (it, h) if hist else it

    def pcg_omp(self, r, x, tol, maxit, precond=1, fixed=False):
        """BPPCG on all host threads (the CPU timing baseline), its operator
        from the CPU baseline build (cpu_axhelm.c): returns (iterations, set-up
        seconds)."""
        fn = C.cast(cpu_lib().nekbc_axhelm, C.c_void_p)
        lib().nekbo_set_cpu_axhelm(fn)
        setup = C.c_double(0.0)
        it = lib().nekbo_pcg_omp(C.byref(self.s), r, x, tol, maxit, precond, int(fixed),
                                 C.byref(setup))
        return it, setup.value


def zero_mean(q, Nloc, Nfields=1, offset=None):
    """BPZeroMean restatement, in place on the float64 array q."""
    offset = Nloc if offset is None else offset
    lib().nekbo_zero_mean(Nloc, Nfields, offset, q)
    return q


# ----------------------------------------------------------------------------- dot, adv
def dot_partials(variant, w, x, y, N=None, Nfields=1, offset=0, block_size=256):
    """Per-block partials of the dot benchmark kernels (dot/kernel/VOLTA/dot.okl)."""
    N = w.size if N is None and Nfields == 1 else N
    out = np.zeros(max(1, -(-N // block_size)), dtype=np.float64)
    nb = lib().nekbo_dot_partials(variant, N, Nfields, offset, block_size,
                                  *(np.ascontiguousarray(a, np.float64) for a in (w, x, y)), out)
    if nb < 0:
        raise ValueError("dot: bad arguments")
    return out[:nb]


def adv_cubature(Nq, cubNq, E, vgeo, cubvgeo, cubD, cubInterpT, U, offset=None):
    """advCubatureHex3D_v0 restatement (adv/kernel/VOLTA/adv.okl:27-261)."""
    offset = E * Nq ** 3 if offset is None else offset
    NU = np.zeros(3 * offset, dtype=np.float64)
    args = [np.ascontiguousarray(a, np.float64) for a in (vgeo, cubvgeo, cubD, cubInterpT)]
    lib().nekbo_adv_cubature(Nq, cubNq, E, *args, offset, np.ascontiguousarray(U, np.float64), NU)
    return NU


# ----------------------------------------------------------------------------- conv net
def conv3d_forward(Nq, W, x, Cin, Cout):
    E = x.size // (Cin * Nq ** 3)
    out = np.zeros(E * Cout * Nq ** 3, dtype=np.float32)
    lib().nekbo_conv3d_forward(Nq, E, Cin, Cout, np.ascontiguousarray(W, np.float32),
                               np.ascontiguousarray(x, np.float32), out)
    return out


def conv3d_backward(Nq, W, x, gout, Cin, Cout, want_gin=True):
    E = x.size // (Cin * Nq ** 3)
    gin = np.zeros(E * Cin * Nq ** 3, dtype=np.float32) if want_gin else None
    gW = np.zeros(Cout * Cin * 27, dtype=np.float32)
    lib().nekbo_conv3d_backward(Nq, E, Cin, Cout, np.ascontiguousarray(W, np.float32),
                                np.ascontiguousarray(x, np.float32),
                                np.ascontiguousarray(gout, np.float32), _ptr(gin), gW)
    return gin, gW


def gelu(x):
    x = np.ascontiguousarray(x, np.float32)
    y = np.empty_like(x)
    lib().nekbo_gelu_forward(x.size, x, y)
    return y


def gelu_backward(x, gy):
    x = np.ascontiguousarray(x, np.float32)
    gx = np.empty_like(x)
    lib().nekbo_gelu_backward(x.size, x, np.ascontiguousarray(gy, np.float32), gx)
    return gx


def net_forward(Nq, W, x, C):
    """3-layer element network 1 -> C -> C -> 1 with GELU after layers 1 and 2;
    W = [W1 (C,1,27), W2 (C,C,27), W3 (1,C,27)] flattened."""
    o2, o3 = 27 * C, 27 * C + 27 * C * C
    z1 = conv3d_forward(Nq, W[:o2], x, 1, C)
    a1 = gelu(z1)
    z2 = conv3d_forward(Nq, W[o2:o3], a1, C, C)
    a2 = gelu(z2)
    y = conv3d_forward(Nq, W[o3:], a2, C, 1)
    return y, (z1, a1, z2, a2)


def net_loss_grad(Nq, W, x, t, C):
    """loss = mean (net(x) - t)^2 and its gradient w.r.t. W, by the chain rule
    through the oracle's layer backward passes."""
    o2, o3 = 27 * C, 27 * C + 27 * C * C
    y, (z1, a1, z2, a2) = net_forward(Nq, W, x, C)
    d = y.astype(np.float64) - t
    loss = float(np.mean(d * d))
    gy = (2 * d / d.size).astype(np.float32)
    ga2, gW3 = conv3d_backward(Nq, W[o3:], a2, gy, C, 1)
    gz2 = gelu_backward(z2, ga2)
    ga1, gW2 = conv3d_backward(Nq, W[o2:o3], a1, gz2, C, C)
    gz1 = gelu_backward(z1, ga1)
    _, gW1 = conv3d_backward(Nq, W[:o2], x, gz1, 1, C, want_gin=False)
    return loss, np.concatenate([gW1, gW2, gW3])


# ----------------------------------------------------------------------------- reference shims
_CPU = None


def cpu_lib():
    """The timed CPU baseline (cpu_axhelm.c): the reference's CPU axhelm with the
    order fixed at compile time and the reference's -O3."""
    global _CPU
    if _CPU is None:
        path = os.path.join(_HERE, "libcpuaxhelm.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.nekbc_axhelm.restype = C.c_int
        L.nekbc_axhelm.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_int64, _d, _d, _vp, _d, _d]
        _CPU = L
    return _CPU


def cpu_axhelm(Nq, bk, E, offset, ggeo, D, lam, q, Aq):
    """Single-field axhelm on E elements with the CPU baseline (OpenMP)."""
    lp = None if lam is None else np.ascontiguousarray(lam, dtype=np.float64)
    rc = cpu_lib().nekbc_axhelm(Nq, int(bool(bk)), E, offset, ggeo, D,
                                None if lp is None else lp.ctypes.data, q, Aq)
    if rc != 0:
        raise ValueError(f"CPU baseline: Nq={Nq} outside 2..14")
    return Aq


def ref(Nq: int, fast: bool = False):
    """The reference's own CPU axhelm compiled for this Nq, or None when not
    built; ``fast``: the build with the reference's own flags (make ref-fast)."""
    key = (Nq, fast)
    if key in _REFS:
        return _REFS[key]
    path = os.path.join(_HERE, "_ref", f"libnekref_{'fast_' if fast else ''}nq{Nq}.so")
    if not os.path.exists(path):
        _REFS[key] = None
        return None
    L = C.CDLL(path)
    L.nekref_nq.restype = C.c_int
    L.nekref_axhelm_reference.argtypes = [C.c_int, C.c_int, C.c_double, _d, _d, _d, _d]
    L.nekref_axhelm_cpu.restype = C.c_int
    L.nekref_axhelm_cpu.argtypes = [C.c_int, C.c_int, C.c_int, _d, _d, _vp, _d, _d]
    L.nekref_weighted_inner_product_update.argtypes = [C.c_int, C.c_int, _d, _d, _d, _d]
    _REFS[key] = L
    return L
