"""GB300-native spectral-element hot path of nekBench (axhelm, gather-scatter, PCG).

Python front end over the C ABI of ``libnekb_gb300.so`` (see ``include/nekb.h``).
It mirrors the reference's host interface for this path:

* ``load_ax_kernel(name, N)`` returns a callable with the OCCA kernel's argument
  order ``kernel(Nelements, offset, ggeo, D, lambda, q, Aq)`` (as built by
  ``loadAxKernel``, axhelm/kernelHelper.cpp:3-58, and launched at
  nekBone/solve.cpp:218, axhelm/main.cpp:132);
* ``ogs_setup(ids)`` / ``OGS.gather_scatter_many(v, k, stride, type, op)``
  mirror ``ogsSetup`` and ``ogsGatherScatterMany`` (3rdParty/ogs/ogs.hpp:178,200);
* ``BP`` holds a box-mesh benchmark problem and ``BP.pcg`` mirrors ``BPPCG``
  (nekBone/solve.cpp:44-113).

Device arrays are torch CUDA tensors (torch supplies device memory and streams
only; every computation runs in this package's own kernels).  There is no CPU
fallback: without the CUDA library or a GPU every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnekb_gb300.so")

AX_BK, AX_N3, AX_PARTIAL = 1, 2, 4
FP64, FP32, BF16, FP32_TRILINEAR, FP64_SPLIT = 0, 1, 2, 3, 4
DOUBLE, FLOAT = 0, 1
PRECOND_COPY, PRECOND_JACOBI, PRECOND_LEARNED = 0, 1, 2
SOLVER_FP64, SOLVER_MIXED, SOLVER_FP64_SPLIT = 0, 1, 2
NET_FP32, NET_TENSOR, NET_TENSOR_SYNC, NET_TENSOR_TC5 = 0, 1, 2, 3
OK, ERR_INVALID, ERR_CUDA, ERR_ALLOC, ERR_UNSUPPORTED, ERR_BREAKDOWN, ERR_NOT_CONVERGED = \
    0, -1, -2, -3, -4, -5, -6

EXPORTED = [
    "nekb_last_error", "nekb_version", "nekb_device_sync", "nekb_copy", "nekb_axhelm",
    "nekb_axhelm_flags_from_name", "nekb_update_jacobi", "nekb_geometric_factors",
    "nekb_trilinear_coeffs", "nekb_gll", "nekb_gauss", "nekb_dmatrix", "nekb_fill_uniform",
    "nekb_ogs_setup", "nekb_ogs_free", "nekb_ogs_gs_many", "nekb_ogs_sizes", "nekb_ogs_copy_csr",
    "nekb_ogs_inv_degree", "nekb_mask", "nekb_bp_setup", "nekb_bp_setup_mesh", "nekb_bp_free",
    "nekb_bp_sizes",
    "nekb_bp_device_ptr", "nekb_bp_ogs", "nekb_bp_apply", "nekb_bp_weighted_inner_product",
    "nekb_bp_weighted_inner_product2", "nekb_weighted_inner_product_noalloc",
    "nekb_pcg_default_opts", "nekb_bp_pcg", "nekb_bp_zero_mean", "nekb_bp_local_correction",
    "nekb_net_create", "nekb_net_free", "nekb_net_set_inference", "nekb_net_inference",
    "nekb_net_num_params", "nekb_net_get_weights",
    "nekb_net_set_weights", "nekb_net_forward", "nekb_net_raise_copy_timeout", "nekb_net_train_step", "nekb_net_gradient",
    "nekb_net_prepare_pairs", "nekb_net_save", "nekb_net_load", "nekb_peak_fma", "nekb_peak_copy",
    "nekb_dot_num_blocks", "nekb_dot_partials", "nekb_adv_cubature",
]


class NekbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"nekb error {code}: {msg}")
        self.code = code


class BPConfig(C.Structure):
    _fields_ = [("N", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("Nfields", C.c_int), ("periodic", C.c_int), ("dirichlet", C.c_int),
                ("perturb", C.c_double), ("seed", C.c_uint64), ("box_min", C.c_double),
                ("box_max", C.c_double)]


class PcgOpts(C.Structure):
    _fields_ = [("solver", C.c_int), ("precond", C.c_int), ("flexible", C.c_int),
                ("fixed_iterations", C.c_int), ("bk", C.c_int), ("inner_precision", C.c_int),
                ("inner_tol", C.c_double), ("max_outer", C.c_int), ("check_every", C.c_int),
                ("use_graph", C.c_int), ("net", C.c_void_p), ("zero_mean", C.c_int),
                ("fcg_window", C.c_int)]


class PcgStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("outer_iterations", C.c_int), ("status", C.c_int),
                ("rdotr0", C.c_double), ("rdotr", C.c_double), ("true_rel_res", C.c_double),
                ("elapsed_s", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    """The loaded C library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise NekbError(ERR_UNSUPPORTED, f"{LIB_PATH} not built: run nekbench_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    vp, i64, i32, d = C.c_void_p, C.c_int64, C.c_int, C.c_double
    L.nekb_last_error.restype = C.c_char_p
    L.nekb_copy.argtypes = [vp, vp, i64]
    L.nekb_axhelm.argtypes = [i32, i32, i32, i64, i64, vp, vp, vp, vp, vp, vp, vp]
    L.nekb_axhelm_flags_from_name.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
    L.nekb_update_jacobi.argtypes = [i32, i64, i64, vp, vp, vp, vp, vp, vp]
    L.nekb_geometric_factors.argtypes = [i32, i64, vp, vp, vp, vp, vp, vp, vp]
    L.nekb_trilinear_coeffs.argtypes = [i64, vp, vp, vp, vp, vp]
    L.nekb_gll.argtypes = [i32, vp, vp]
    L.nekb_gauss.argtypes = [i32, vp, vp]
    L.nekb_dmatrix.argtypes = [i32, vp, vp]
    L.nekb_fill_uniform.argtypes = [vp, i64, C.c_uint64, C.c_uint64, d, d, vp]
    L.nekb_ogs_setup.restype = vp
    L.nekb_ogs_setup.argtypes = [i64, vp, i32, C.POINTER(C.c_int)]
    L.nekb_ogs_free.argtypes = [vp]
    L.nekb_ogs_gs_many.argtypes = [vp, vp, i32, i64, i32, i32, vp]
    L.nekb_ogs_sizes.argtypes = [vp, vp]
    L.nekb_ogs_copy_csr.argtypes = [vp, vp, vp]
    L.nekb_ogs_inv_degree.restype = vp
    L.nekb_ogs_inv_degree.argtypes = [vp]
    L.nekb_mask.argtypes = [i64, vp, vp, i32, vp]
    L.nekb_bp_setup.restype = vp
    L.nekb_bp_setup.argtypes = [C.POINTER(BPConfig), vp, C.POINTER(C.c_int)]
    L.nekb_bp_setup_mesh.restype = vp
    L.nekb_bp_setup_mesh.argtypes = [i32, i64, i32, vp, vp, i64, vp, vp, vp, vp, vp,
                                     C.POINTER(C.c_int)]
    L.nekb_bp_free.argtypes = [vp]
    L.nekb_bp_sizes.argtypes = [vp, vp]
    L.nekb_bp_device_ptr.restype = vp
    L.nekb_bp_device_ptr.argtypes = [vp, C.c_char_p]
    L.nekb_bp_ogs.restype = vp
    L.nekb_bp_ogs.argtypes = [vp]
    L.nekb_bp_apply.argtypes = [vp, i32, i32, vp, vp, vp]
    L.nekb_bp_weighted_inner_product.argtypes = [vp, vp, vp, vp, vp]
    L.nekb_bp_weighted_inner_product2.argtypes = [vp, vp, vp, vp, vp]
    L.nekb_pcg_default_opts.argtypes = [C.POINTER(PcgOpts)]
    L.nekb_bp_pcg.argtypes = [vp, vp, vp, vp, d, i32, C.POINTER(PcgOpts), C.POINTER(PcgStats)]
    L.nekb_bp_zero_mean.argtypes = [vp, vp]
    L.nekb_dot_num_blocks.restype = i64
    L.nekb_dot_num_blocks.argtypes = [i64, i32]
    L.nekb_dot_partials.argtypes = [i32, i64, i32, i64, i32, vp, vp, vp, vp, vp]
    L.nekb_adv_cubature.argtypes = [i32, i32, i32, i64, vp, vp, vp, vp, i64, vp, vp, vp]
    if hasattr(L, "nekb_net_create"):
        L.nekb_net_create.restype = vp
        L.nekb_net_create.argtypes = [i32, i32, i32, C.c_uint64, C.POINTER(C.c_int)]
        L.nekb_net_free.argtypes = [vp]
        L.nekb_net_set_inference.argtypes = [vp, i32]
        L.nekb_net_inference.argtypes = [vp]
        L.nekb_net_num_params.argtypes = [vp]
        L.nekb_net_get_weights.argtypes = [vp, vp]
        L.nekb_net_set_weights.argtypes = [vp, vp]
        L.nekb_net_forward.argtypes = [vp, i64, vp, vp, vp]
        L.nekb_net_raise_copy_timeout.argtypes = []
        L.nekb_net_train_step.argtypes = [vp, i64, vp, vp, C.c_float, vp, vp]
        L.nekb_net_gradient.argtypes = [vp, i64, vp, vp, vp, vp, vp]
        L.nekb_net_prepare_pairs.argtypes = [i32, i64, i64, vp, vp, vp, vp, vp, vp]
        L.nekb_bp_local_correction.argtypes = [vp, vp, vp, i64, vp, vp, vp, i32, C.c_float]
        L.nekb_net_save.argtypes = [vp, C.c_char_p]
        L.nekb_net_load.restype = vp
        L.nekb_net_load.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
    L.nekb_peak_fma.argtypes = [i32, vp]
    L.nekb_peak_copy.argtypes = [vp]
    _lib = L
    return L


def check(code):
    if code != OK:
        raise NekbError(code, lib().nekb_last_error().decode())
    return code


def check_value(v):
    """A non-negative return value, or the error it encodes."""
    if v < 0:
        raise NekbError(v, lib().nekb_last_error().decode())
    return v


def _ptr(t):
    if t is None:
        return None
    if isinstance(t, int):
        return t
    return t.data_ptr()


def _stream(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return stream


def _order_after_torch():
    """The problem's entry points run on its own stream: wait for the work that
    torch has queued on its current stream (the producers of their inputs)."""
    import torch
    if torch.cuda.is_available() and torch.cuda.is_initialized():
        torch.cuda.current_stream().synchronize()


def _require_cuda(*ts):
    for t in ts:
        if t is not None and not isinstance(t, int) and not t.is_cuda:
            raise NekbError(ERR_INVALID, "device arrays must be CUDA tensors")


# --------------------------------------------------------------------------- axhelm
def flags_from_name(name: str) -> int:
    f = C.c_int(0)
    check(lib().nekb_axhelm_flags_from_name(name.encode(), C.byref(f)))
    return f.value


def axhelm(Nq, flags, precision, Nelements, offset, ggeo, D, lam, q, Aq, element_list=None,
           stream=None):
    """One axhelm application (device tensors)."""
    _require_cuda(ggeo, D, lam, q, Aq, element_list)
    check(lib().nekb_axhelm(Nq, flags, precision, Nelements, offset, _ptr(element_list), _ptr(ggeo),
                            _ptr(D), _ptr(lam), _ptr(q), _ptr(Aq), _stream(stream)))


def load_ax_kernel(name: str, N: int, precision: int = FP64):
    """Kernel object with the OCCA argument order of ``loadAxKernel``'s result."""
    flags = flags_from_name(name)
    Nq = N + 1

    if flags & AX_PARTIAL:
        def kernel(Nelements, offset, elementList, ggeo, D, lam, q, Aq):
            axhelm(Nq, flags, precision, Nelements, offset, ggeo, D, lam, q, Aq, elementList)
    else:
        def kernel(Nelements, offset, ggeo, D, lam, q, Aq):
            axhelm(Nq, flags, precision, Nelements, offset, ggeo, D, lam, q, Aq)
    kernel.flags, kernel.Nq, kernel.name = flags, Nq, name
    return kernel


def update_jacobi(Nq, Nelements, offset, mapB, ggeo, D, lam, diag, stream=None):
    check(lib().nekb_update_jacobi(Nq, Nelements, offset, _ptr(mapB), _ptr(ggeo), _ptr(D),
                                   _ptr(lam), _ptr(diag), _stream(stream)))


def geometric_factors(Nq, E, EX, EY, EZ, r1d, w1d, ggeo, stream=None):
    import numpy as np
    r = np.ascontiguousarray(r1d, dtype=np.float64)
    w = np.ascontiguousarray(w1d, dtype=np.float64)
    check(lib().nekb_geometric_factors(Nq, E, _ptr(EX), _ptr(EY), _ptr(EZ), r.ctypes.data,
                                       w.ctypes.data, _ptr(ggeo), _stream(stream)))


def trilinear_coeffs(E, EX, EY, EZ, coef, stream=None):
    check(lib().nekb_trilinear_coeffs(E, _ptr(EX), _ptr(EY), _ptr(EZ), _ptr(coef), _stream(stream)))


def gll(N):
    import numpy as np
    r, w = np.zeros(N + 1), np.zeros(N + 1)
    check(lib().nekb_gll(N, r.ctypes.data, w.ctypes.data))
    return r, w


def gauss(N):
    import numpy as np
    r, w = np.zeros(N + 1), np.zeros(N + 1)
    check(lib().nekb_gauss(N, r.ctypes.data, w.ctypes.data))
    return r, w


def dmatrix(r):
    import numpy as np
    r = np.ascontiguousarray(r, dtype=np.float64)
    D = np.zeros(len(r) * len(r))
    check(lib().nekb_dmatrix(len(r), r.ctypes.data, D.ctypes.data))
    return D


def fill_uniform(v, seed, stream_id, lo=0.0, hi=1.0, stream=None):
    check(lib().nekb_fill_uniform(_ptr(v), v.numel(), seed, stream_id, lo, hi, _stream(stream)))
    return v


# --------------------------------------------------------------------------- gather-scatter
class OGS:
    """Gather-scatter handle (ogsSetup / ogsGatherScatterMany on one rank)."""

    def __init__(self, ids, verbose=0, _handle=None, _owner=None):
        import numpy as np
        self._owner = _owner
        if _handle is not None:
            self.h = _handle
            self._owned = False
        else:
            ids = np.ascontiguousarray(ids, dtype=np.int64)
            st = C.c_int(0)
            self.h = lib().nekb_ogs_setup(len(ids), ids.ctypes.data, verbose, C.byref(st))
            check(st.value)
            self._owned = True
        s = (C.c_int64 * 4)()
        check(lib().nekb_ogs_sizes(self.h, s))
        self.N, self.Nlocal, self.NlocalGather, self.Nmulti = list(s)

    def gather_scatter_many(self, v, k=1, stride=0, type="double", op="add", stream=None):
        _require_cuda(v)
        dt = {"double": DOUBLE, "float": FLOAT}[type]
        if op != "add":
            raise NekbError(ERR_UNSUPPORTED, "only the add operation is supported")
        check(lib().nekb_ogs_gs_many(self.h, _ptr(v), k, stride, dt, 0, _stream(stream)))

    def csr(self):
        import numpy as np
        offs = np.zeros(self.NlocalGather + 1, dtype=np.int32)
        ids = np.zeros(max(self.Nlocal, 1), dtype=np.int32)
        check(lib().nekb_ogs_copy_csr(self.h, offs.ctypes.data, ids.ctypes.data))
        return offs, ids[: self.Nlocal]

    def inv_degree(self):
        """invDegree as a torch tensor view of the handle's device array (copied)."""
        import torch
        p = lib().nekb_ogs_inv_degree(self.h)
        out = torch.empty(self.N, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _cuda_memcpy(out.data_ptr(), p, self.N * 8)
        return out

    def free(self):
        if self.h and self._owned:
            lib().nekb_ogs_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def ogs_setup(ids, verbose=0):
    return OGS(ids, verbose)


def mask(mask_ids, q, dtype=DOUBLE, stream=None):
    check(lib().nekb_mask(mask_ids.numel(), _ptr(mask_ids), _ptr(q), dtype, _stream(stream)))


def _cuda_memcpy(dst, src, nbytes):
    check(lib().nekb_copy(C.c_void_p(dst), C.c_void_p(src), nbytes))


# --------------------------------------------------------------------------- benchmark problem
class BP:
    """Box-mesh benchmark problem on the device (mesh_t + BP_t of nekBone)."""

    def __init__(self, N, nx, ny=None, nz=None, Nfields=1, periodic=False, dirichlet=True,
                 perturb=0.1, seed=1, stream=None, box=(0.0, 0.0)):
        """box=(lo, hi): the cube [lo, hi]^3; (0, 0) is the unit cube."""
        ny = nx if ny is None else ny
        nz = nx if nz is None else nz
        self.cfg = BPConfig(N, nx, ny, nz, Nfields, int(periodic), int(dirichlet), perturb, seed,
                            float(box[0]), float(box[1]))
        st = C.c_int(0)
        self.h = lib().nekb_bp_setup(C.byref(self.cfg), stream, C.byref(st))
        check(st.value)
        s = (C.c_int64 * 6)()
        check(lib().nekb_bp_sizes(self.h, s))
        self.Nq, self.E, self.Np, self.offset, self.Nmasked, self.Nfields = list(s)
        self.N = N
        self.Nlocal = self.E * self.Np
        self.ogs = OGS(None, _handle=lib().nekb_bp_ogs(self.h), _owner=self)

    @classmethod
    def from_mesh(cls, N, Nelements, ggeo, ids, mask_ids=None, EX=None, EY=None, EZ=None,
                  Nfields=1, stream=None):
        """Problem on the caller's mesh (ggeo device/host FP64 in the reference
        layout, global ids host int64, masked node list host int32, optional
        8 vertices per element)."""
        import numpy as np
        self = cls.__new__(cls)
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        mk = np.ascontiguousarray(mask_ids if mask_ids is not None else np.zeros(0), dtype=np.int32)
        vx = [None if v is None else np.ascontiguousarray(v, dtype=np.float64) for v in (EX, EY, EZ)]
        gp = ggeo.data_ptr() if hasattr(ggeo, "data_ptr") else \
            np.ascontiguousarray(ggeo, dtype=np.float64).ctypes.data
        self._keep = (ggeo, ids, mk, vx)
        st = C.c_int(0)
        self.h = lib().nekb_bp_setup_mesh(
            N, Nelements, Nfields, gp, ids.ctypes.data, len(mk),
            mk.ctypes.data if len(mk) else None,
            *[v.ctypes.data if v is not None else None for v in vx], stream, C.byref(st))
        check(st.value)
        s = (C.c_int64 * 6)()
        check(lib().nekb_bp_sizes(self.h, s))
        self.Nq, self.E, self.Np, self.offset, self.Nmasked, self.Nfields = list(s)
        self.N = N
        self.Nlocal = self.E * self.Np
        self.ogs = OGS(None, _handle=lib().nekb_bp_ogs(self.h), _owner=self)
        return self

    def device_array(self, name, n, dtype):
        """Copy of a device array owned by the problem, as a torch tensor."""
        import torch
        p = lib().nekb_bp_device_ptr(self.h, name.encode())
        if not p:
            raise NekbError(ERR_INVALID, lib().nekb_last_error().decode())
        out = torch.empty(n, dtype=dtype, device="cuda")
        torch.cuda.synchronize()
        _cuda_memcpy(out.data_ptr(), p, n * out.element_size())
        return out

    def ptr(self, name):
        p = lib().nekb_bp_device_ptr(self.h, name.encode())
        if not p:
            raise NekbError(ERR_INVALID, lib().nekb_last_error().decode())
        return p

    def weighted_inner_product(self, w, a, b):
        """BPWeightedInnerProduct: sum over fields of w a b (host float)."""
        out = C.c_double(0)
        _order_after_torch()
        check(lib().nekb_bp_weighted_inner_product(self.h, _ptr(w), _ptr(a), _ptr(b),
                                                   C.byref(out)))
        return out.value

    def weighted_inner_product2(self, w, a, b):
        """BPWeightedInnerProduct2: (sum w a b, sum w a a)."""
        out = (C.c_double * 2)()
        _order_after_torch()
        check(lib().nekb_bp_weighted_inner_product2(self.h, _ptr(w), _ptr(a), _ptr(b), out))
        return out[0], out[1]

    def zero_mean(self, q):
        """BPZeroMean: subtract the mean of the local values over all fields."""
        _order_after_torch()
        check(lib().nekb_bp_zero_mean(self.h, _ptr(q)))

    def apply(self, q, Aq, lam=None, bk=False, precision=FP64):
        _order_after_torch()
        check(lib().nekb_bp_apply(self.h, int(bk), precision, _ptr(lam), _ptr(q), _ptr(Aq)))

    def local_correction(self, lam, elems, r, inv_diag, y, iters=200, tol=1e-5):
        """Element-interior Helmholtz solve of residual rows r [n, Np] (float32,
        row b from element elems[b], int32) with the Jacobi value invDiag*r on
        the element-boundary nodes; result in y."""
        n = int(elems.numel())
        _order_after_torch()
        check(lib().nekb_bp_local_correction(self.h, _ptr(lam), _ptr(elems), n, _ptr(r),
                                             _ptr(inv_diag), _ptr(y), int(iters), float(tol)))

    def pcg(self, lam, r, x, tol, maxit, solver=SOLVER_FP64, precond=PRECOND_JACOBI,
            flexible=False, fixed_iterations=False, bk=False, inner_precision=FP32,
            inner_tol=1e-2, max_outer=40, check_every=16, use_graph=True, net=None,
            zero_mean=False, fcg_window=0):
        """BPPCG: r (rhs in, residual out) and x (guess in, solution out) are device FP64;
        zero_mean: BPZeroMean on r before and on x after, as solve() does for an
        all-Neumann problem."""
        o = PcgOpts()
        lib().nekb_pcg_default_opts(C.byref(o))
        o.solver, o.precond, o.flexible, o.fixed_iterations, o.bk = \
            solver, precond, int(flexible), int(fixed_iterations), int(bk)
        o.inner_precision, o.inner_tol, o.max_outer = inner_precision, inner_tol, max_outer
        o.check_every, o.use_graph = check_every, int(use_graph)
        o.net = net.h if net is not None else None
        o.zero_mean = int(zero_mean)
        o.fcg_window = int(fcg_window)
        st = PcgStats()
        _order_after_torch()
        check(lib().nekb_bp_pcg(self.h, _ptr(lam), _ptr(r), _ptr(x), tol, maxit, C.byref(o),
                                C.byref(st)))
        return st.as_dict()

    def free(self):
        if getattr(self, "h", None):
            lib().nekb_bp_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Net:
    """Learned element preconditioner (3 layers of 3x3x3 convolutions per element)."""

    def __init__(self, Nq=8, channels=16, layers=3, seed=1, _handle=None):
        if _handle is not None:
            self.h = _handle
        else:
            st = C.c_int(0)
            self.h = lib().nekb_net_create(Nq, channels, layers, seed, C.byref(st))
            check(st.value)
        self.P = lib().nekb_net_num_params(self.h)

    @classmethod
    def load(cls, path):
        st = C.c_int(0)
        h = lib().nekb_net_load(os.fsencode(path), C.byref(st))
        check(st.value)
        return cls(_handle=h)

    def save(self, path):
        check(lib().nekb_net_save(self.h, os.fsencode(path)))

    def weights(self):
        import numpy as np
        w = np.zeros(self.P, dtype=np.float32)
        check(lib().nekb_net_get_weights(self.h, w.ctypes.data))
        return w

    def set_weights(self, w):
        import numpy as np
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == self.P
        check(lib().nekb_net_set_weights(self.h, w.ctypes.data))

    @property
    def inference(self):
        """NET_TENSOR (BF16 tensor-core MMAs, the library's kernel), NET_TENSOR_SYNC
        (mma.sync), NET_TENSOR_TC5 (tcgen05) or NET_FP32 (CUDA cores), as used."""
        return check_value(lib().nekb_net_inference(self.h))

    @inference.setter
    def inference(self, mode):
        check(lib().nekb_net_set_inference(self.h, int(mode)))

    def forward(self, inp, out, E, stream=None):
        check(lib().nekb_net_forward(self.h, E, _ptr(inp), _ptr(out), _stream(stream)))

    def gradient(self, inp, target, E, stream=None):
        import numpy as np
        g = np.zeros(self.P, dtype=np.float32)
        loss = C.c_float(0)
        check(lib().nekb_net_gradient(self.h, E, _ptr(inp), _ptr(target), g.ctypes.data,
                                      C.byref(loss), _stream(stream)))
        return g, loss.value

    def train_step(self, inp, target, E, lr, stream=None):
        loss = C.c_float(0)
        check(lib().nekb_net_train_step(self.h, E, _ptr(inp), _ptr(target), C.c_float(lr),
                                        C.byref(loss), _stream(stream)))
        return loss.value

    def free(self):
        if getattr(self, "h", None):
            lib().nekb_net_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def prepare_pairs(Np, E, Efield, r, err, inv_diag, inp, target, stream=None):
    check(lib().nekb_net_prepare_pairs(Np, E, Efield, _ptr(r), _ptr(err), _ptr(inv_diag),
                                       _ptr(inp), _ptr(target), _stream(stream)))


# --------------------------------------------------------------------------- dot, adv
DOT_V0, DOT_V1, DOT_BLOCK = 0, 1, 2
_DOT_NAMES = {"weightedInnerProduct2_v0": DOT_V0, "weightedInnerProduct2_v1": DOT_V1,
              "weightedBlockInnerProduct2": DOT_BLOCK}


def dot_num_blocks(N, block_size=256):
    return check_value(lib().nekb_dot_num_blocks(N, block_size))


def dot_partials(variant, N, w, x, y, wxy, Nfields=1, offset=0, block_size=256, stream=None):
    """Per-block partials of the dot benchmark kernels (dot/kernel/VOLTA/dot.okl)."""
    _require_cuda(w, x, y, wxy)
    check(lib().nekb_dot_partials(variant, N, Nfields, offset, block_size, _ptr(w), _ptr(x), _ptr(y),
                                  _ptr(wxy), _stream(stream)))


def load_dot_kernel(name: str, block_size: int = 256, Nfields: int = 1):
    """Kernel object with the argument order of the dot driver's kernel
    (dot/main.cpp:31): ``kernel(N, w, x, y, wxy)``; weightedBlockInnerProduct2
    takes ``kernel(N, offset, w, x, y, wxy)`` (dot.okl:67)."""
    if name not in _DOT_NAMES:
        raise NekbError(ERR_INVALID, f"unknown dot kernel {name!r}")
    variant = _DOT_NAMES[name]
    if variant == DOT_BLOCK:
        def kernel(N, offset, w, x, y, wxy):
            dot_partials(variant, N, w, x, y, wxy, Nfields, offset, block_size)
    else:
        def kernel(N, w, x, y, wxy):
            dot_partials(variant, N, w, x, y, wxy, 1, 0, block_size)
    kernel.variant, kernel.block_size, kernel.name = variant, block_size, name
    return kernel


def adv_cubature(Nq, cubNq, Nelements, vgeo, cubvgeo, cubD, cubInterpT, offset, U, NU,
                 precision=FP64, stream=None):
    """advCubatureHex3D_v0 (adv/kernel/VOLTA/adv.okl:27) on device tensors;
    precision FP64 or FP64_SPLIT (double-float arithmetic on the FP32 pipes)."""
    _require_cuda(vgeo, cubvgeo, cubD, cubInterpT, U, NU)
    check(lib().nekb_adv_cubature(Nq, cubNq, precision, Nelements, _ptr(vgeo), _ptr(cubvgeo),
                                  _ptr(cubD), _ptr(cubInterpT), offset, _ptr(U), _ptr(NU),
                                  _stream(stream)))


def load_adv_kernel(N: int, cubN: int, precision: int = FP64):
    """Kernel object with the adv driver's argument order (adv/main.cpp:115-123):
    ``kernel(Nelements, vgeo, cubvgeo, cubD, cubInterpT, offset, U, NU)``."""
    Nq, cubNq = N + 1, cubN + 1

    def kernel(Nelements, vgeo, cubvgeo, cubD, cubInterpT, offset, U, NU):
        adv_cubature(Nq, cubNq, Nelements, vgeo, cubvgeo, cubD, cubInterpT, offset, U, NU,
                     precision)
    kernel.Nq, kernel.cubNq, kernel.name = Nq, cubNq, "advCubatureHex3D_v0"
    return kernel


def peak_fma(fp64=True):
    v = C.c_double(0)
    check(lib().nekb_peak_fma(int(fp64), C.byref(v)))
    return v.value


def peak_copy():
    v = C.c_double(0)
    check(lib().nekb_peak_copy(C.byref(v)))
    return v.value
