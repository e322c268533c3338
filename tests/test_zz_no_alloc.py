"""The no-allocation weighted inner product against the regular one.

nekb_weighted_inner_product_noalloc serves callers that cannot call cudaMalloc
(an application whose device memory all belongs to its own pool allocator, or
a time-critical loop that must not trigger cudaMalloc's implicit
synchronisation).  Its scratch is a fixed array inside the library.  This test
calls it through the C ABI twice in a row and compares each result with
nekb_bp_weighted_inner_product (the problem-owned scratch), within the
tolerance the other inner-product tests use; it also checks that a size beyond
the fixed scratch is refused with an error instead of being run.  The file
name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_noalloc_matches_regular_entry_twice(nb, O, dev):
    L = nb.lib()
    L.nekb_weighted_inner_product_noalloc.argtypes = [C.c_int64, C.c_int, C.c_int64, C.c_void_p,
                                                      C.c_void_p, C.c_void_p, C.c_void_p,
                                                      C.c_void_p]
    bp = nb.BP(7, 6, 5, 4, Nfields=3, perturb=0.1, seed=4)
    N, off = bp.Nlocal, bp.offset
    w = bp.ogs.inv_degree()
    out = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):  # two calls in a row share the fixed scratch
        a = torch.from_numpy(O.uniform(3 * N, 30 + call, 1, -1, 1)).to(dev)
        b = torch.from_numpy(O.uniform(3 * N, 30 + call, 2, -1, 1)).to(dev)
        torch.cuda.synchronize()
        rc = L.nekb_weighted_inner_product_noalloc(N, 3, off, w.data_ptr(), a.data_ptr(),
                                                   b.data_ptr(), out.data_ptr(), stream)
        assert rc == nb.OK, L.nekb_last_error()
        torch.cuda.synchronize()
        got = float(out.item())
        ref = bp.weighted_inner_product(w, a, b)
        assert abs(got - ref) <= 1e-12 * abs(ref), (call, got, ref)
        # independent check on the host
        wn, an, bn = w.cpu().numpy(), a.cpu().numpy(), b.cpu().numpy()
        host = sum(float(np.sum(wn * an[f * N:(f + 1) * N] * bn[f * N:(f + 1) * N]))
                   for f in range(3))
        assert abs(got - host) <= 1e-12 * abs(host)


def test_noalloc_rejects_sizes_beyond_its_scratch(nb, dev):
    L = nb.lib()
    L.nekb_weighted_inner_product_noalloc.argtypes = [C.c_int64, C.c_int, C.c_int64, C.c_void_p,
                                                      C.c_void_p, C.c_void_p, C.c_void_p,
                                                      C.c_void_p]
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    big = (1 << 25) + 1  # one node more than the fixed scratch covers
    rc = L.nekb_weighted_inner_product_noalloc(big, 1, big, out.data_ptr(), out.data_ptr(),
                                               out.data_ptr(), out.data_ptr(), None)
    assert rc == nb.ERR_INVALID
    assert b"exceeds the fixed scratch" in L.nekb_last_error()
