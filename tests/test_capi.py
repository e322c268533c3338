"""CPU checks of the C ABI (no GPU needed): the library loads, exports every
entry point include/nekb.h declares, and its host-only functions and argument
checks behave; nothing here launches a kernel."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import nekbench_gb300 as nb
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "nekb.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nekb_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    L = nb.lib()
    syms = declared_symbols()
    assert len(syms) >= 40
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert set(nb.EXPORTED) >= set(syms)


def test_library_is_built_for_sm103a():
    # the build recipe passes only the sm_103a target
    from nekbench_gb300 import build as B
    assert B.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert os.path.exists(nb.LIB_PATH)


@pytest.mark.parametrize("name,flags", [
    ("axhelm_v0", 0), ("axhelm_bk_v0", 1), ("axhelm_n3_v0", 2), ("axhelm_bk_n3_v0", 3),
    ("axhelmPartial_v0", 4), ("axhelmPartial_bk_v0", 5), ("axhelmPartial_n3_v0", 6),
    ("axhelmPartial_bk_n3_v0", 7), ("axhelm_partial_v0", 4)])
def test_kernel_names(name, flags):
    assert nb.flags_from_name(name) == flags


@pytest.mark.parametrize("bad", ["axhelm", "foo_v0", "axhelm_bk", "axhelm_bk_vx"])
def test_bad_kernel_names(bad):
    with pytest.raises(nb.NekbError):
        nb.flags_from_name(bad)


@pytest.mark.parametrize("N", range(1, 12))
def test_host_basis_matches_oracle(N):
    r, w = nb.gll(N)
    ro, wo = O.gll(N)
    assert np.abs(r - ro).max() < 1e-15 and np.abs(w - wo).max() < 1e-14
    assert np.abs(nb.dmatrix(r) - O.dmatrix(ro)).max() < 1e-12
    g, gw = nb.gauss(N)
    go, gwo = O.gauss(N)
    assert np.abs(g - go).max() < 1e-15 and np.abs(gw - gwo).max() < 1e-14


def test_argument_errors_without_a_launch():
    L = nb.lib()
    # order outside the built range: rejected before any device work
    rc = L.nekb_axhelm(15, 0, nb.FP64, 1, 15 ** 3, None, 1, 1, 1, 1, 1, None)
    assert rc == nb.ERR_UNSUPPORTED
    rc = L.nekb_axhelm(13, 0, nb.FP32, 1, 13 ** 3, None, 1, 1, 1, 1, 1, None)  # FP64 only there
    assert rc == nb.ERR_UNSUPPORTED
    rc = L.nekb_axhelm(8, 0, nb.FP64, -1, 0, None, 1, 1, 1, 1, 1, None)
    assert rc == nb.ERR_INVALID
    rc = L.nekb_axhelm(8, 0, nb.FP64, 1, 512, None, 1, 1, None, 1, 1, None)  # lambda NULL
    assert rc == nb.ERR_INVALID and b"lambda" in L.nekb_last_error()
    rc = L.nekb_axhelm(8, nb.AX_PARTIAL, nb.FP64, 1, 512, None, 1, 1, 1, 1, 1, None)
    assert rc == nb.ERR_INVALID
    rc = L.nekb_axhelm(8, 0, nb.FP64, 2, 512, None, 1, 1, 1, 1, 1, None)  # offset < E*Np
    assert rc == nb.ERR_INVALID
    assert L.nekb_axhelm(8, 0, nb.FP64, 0, 0, None, None, None, None, None, None, None) == nb.OK
    st = C.c_int(0)
    cfg = nb.BPConfig(0, 2, 2, 2, 1, 0, 1, 0.1, 1)
    assert not L.nekb_bp_setup(C.byref(cfg), None, C.byref(st)) and st.value == nb.ERR_UNSUPPORTED
    cfg = nb.BPConfig(7, 2, 2, 2, 2, 0, 1, 0.1, 1)
    assert not L.nekb_bp_setup(C.byref(cfg), None, C.byref(st)) and st.value == nb.ERR_INVALID
    assert not L.nekb_ogs_setup(-1, None, 0, C.byref(st)) and st.value == nb.ERR_INVALID
    assert L.nekb_ogs_gs_many(None, None, 1, 0, 0, 0, None) == nb.ERR_INVALID
    assert not L.nekb_net_create(8, 16, 4, 1, C.byref(st)) and st.value == nb.ERR_UNSUPPORTED
    assert not L.nekb_net_create(12, 16, 3, 1, C.byref(st)) and st.value == nb.ERR_UNSUPPORTED
    assert not L.nekb_net_load(b"/nonexistent/net.bin", C.byref(st)) and st.value == nb.ERR_INVALID
    # dot and adv benchmarks
    assert L.nekb_dot_num_blocks(1000, 256) == 4 and L.nekb_dot_num_blocks(1024, 1024) == 1
    assert L.nekb_dot_num_blocks(1000, 300) == nb.ERR_INVALID
    assert L.nekb_dot_partials(3, 10, 1, 0, 256, 1, 1, 1, 1, None) == nb.ERR_INVALID
    assert L.nekb_dot_partials(1, 10, 1, 0, 512, 1, 1, 1, 1, None) == nb.ERR_INVALID
    assert L.nekb_dot_partials(2, 10, 2, 5, 256, 1, 1, 1, 1, None) == nb.ERR_INVALID  # offset < N
    assert L.nekb_dot_partials(0, 10, 1, 0, 256, None, 1, 1, 1, None) == nb.ERR_INVALID
    assert L.nekb_dot_partials(0, 0, 1, 0, 256, None, None, None, None, None) == nb.OK
    assert L.nekb_adv_cubature(8, 13, 0, 1, 1, 1, 1, 1, 512, 1, 1, None) == nb.ERR_UNSUPPORTED
    assert L.nekb_adv_cubature(11, 17, 0, 1, 1, 1, 1, 1, 1331, 1, 1, None) == nb.ERR_UNSUPPORTED
    assert L.nekb_adv_cubature(8, 12, 0, 2, 1, 1, 1, 1, 512, 1, 1, None) == nb.ERR_INVALID
    assert L.nekb_adv_cubature(8, 12, 0, 1, None, 1, 1, 1, 512, 1, 1, None) == nb.ERR_INVALID
    assert L.nekb_adv_cubature(8, 12, nb.FP32, 1, 1, 1, 1, 1, 512, 1, 1, None) == nb.ERR_UNSUPPORTED
    assert L.nekb_adv_cubature(8, 12, 0, 0, None, None, None, None, 0, None, None, None) == nb.OK


def test_ogs_host_setup_matches_oracle_without_gpu_kernels():
    """The CSR build is host code; its result is checked on the GPU machine too."""
    m = O.BoxMesh(3, 2, 2, 2)
    Ng, offs, gids, invdeg = O.ogs_setup(m.ids)
    assert offs[-1] == np.count_nonzero(m.ids) and Ng > 0


def test_nekbone_summary_formulas_reproduce_the_published_run():
    """The driver's throughput and flop figures follow nekBone/main.cpp:156-177:
    fed the published V100 run (N=7, E=8192, BP5, 5000 iterations in 6.71864 s,
    nekBone/readme.md:43-53) they give its 2.09109 GDOF/s/iter and 393.296
    GFLOP/s."""
    from nekbench_gb300.nekbone import throughput
    gdofs, gbs, gflops = throughput(5000, 7, 8, 8192, 1, True, 6.71864)
    assert abs(gdofs - 2.09109) < 1e-5
    assert abs(gflops - 393.296) < 1e-3
    assert gbs > 0


def test_dot_and_adv_driver_figures():
    """dot: GDOF/s = Nelements N^3 / t and GB/s = 3 Np 8 Nelements / t
    (dot/main.cpp:157-159).  adv: the FP64 flops and bytes counted per element
    at N=7, cubN=11 (interpolation + projection 350,208, derivatives 373,248,
    pointwise 57,024, inverse mass 1,536; 10 cubature slots + IJW + U + NU)."""
    from nekbench_gb300 import adv, dot
    g, b = dot.figures(7, 1000, 2.0)
    assert g == pytest.approx(1000 * 343 / 2.0 / 1e9) and b == pytest.approx(3 * 512 * 8 * 1000 / 2.0 / 1e9)
    assert adv.flops(8, 12) == 350208 + 373248 + 57024 + 1536 == 782016
    assert adv.bytes_moved(8, 12) == 8 * (10 * 1728 + 512 + 6 * 512) == 166912


def test_axhelm_driver_figures_reproduce_the_published_runs():
    """The axhelm driver's figures follow axhelm/main.cpp:161-169: fed the
    published runs (axhelm/readme.md:31,42; N=7, BK, 4000 elements) they give
    the printed GDOF/s, GB/s and GFLOP/s."""
    from nekbench_gb300.axhelm_driver import figures
    g, b, f = figures(7, 4000, 1, True, 0.00018497)
    assert g == pytest.approx(7.41742, abs=1e-5)
    assert b == pytest.approx(797.189, abs=1e-3)
    assert f == pytest.approx(1229.0, abs=0.5)
    g, b, f = figures(7, 4000, 1, True, 0.000351181)
    assert g == pytest.approx(3.90682, abs=1e-5) and b == pytest.approx(419.886, abs=1e-3)
    assert f == pytest.approx(647.324, abs=1e-3)
