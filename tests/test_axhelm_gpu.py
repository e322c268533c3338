"""axhelm on the GPU against the CPU oracle (itself pinned to the reference's
axhelmReference.cpp and kernel/CPU/axhelm.c by tests/test_oracle.py).

Tolerances: FP64 1e-12 relative (max-norm, the reference's own check is a
max-abs difference, axhelm/main.cpp:143-158); FP32 arithmetic 2e-5 relative
against the oracle fed the same rounded inputs; FP32 trilinear geometry 1e-5."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def T(x, dev, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(x))
    return t.to(dev) if dtype is None else t.to(dtype).to(dev)


def bf16_round(x):
    """double -> float32 -> bfloat16 (round to nearest even), as the library converts."""
    f = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (f >> 16) & 1
    r = ((f + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def fields(O, L, nf, seed):
    lam = np.concatenate([O.uniform(L, seed, 1, 0.5, 1.5), O.uniform(L, seed, 2, 0.5, 2.0)])
    q = O.uniform(nf * L, seed, 3, -1, 1)
    return lam, q


@pytest.mark.parametrize("prec", ["FP64", "FP64_SPLIT"])
@pytest.mark.parametrize("N", list(range(1, 14)))
@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_fp64_all_orders_variants(nb, O, dev, N, flags, prec):
    if prec != "FP64" and N > 11:
        with pytest.raises(nb.NekbError):
            nb.axhelm(N + 1, flags, getattr(nb, prec), 1, (N + 1) ** 3,
                      *(torch.zeros(n, dtype=torch.float64, device=dev) for n in
                        (7 * (N + 1) ** 3, (N + 1) ** 2, 2 * (N + 1) ** 3, 3 * (N + 1) ** 3,
                         3 * (N + 1) ** 3)))
        return
    m = O.BoxMesh(N, 3, 2, 2, perturb=0.1, seed=N)  # E=12, not a multiple of the CTA's elements
    E, L = m.E, m.Nlocal
    nf = 3 if flags & nb.AX_N3 else 1
    lam, q = fields(O, L, nf, 100 + N)
    ref = O.axhelm(N + 1, E, L, flags, m.ggeo, m.D, lam, q)
    Aq = torch.zeros(nf * L, dtype=torch.float64, device=dev)
    nb.axhelm(N + 1, flags, getattr(nb, prec), E, L, T(m.ggeo, dev), T(m.D, dev), T(lam, dev),
              T(q, dev), Aq)
    torch.cuda.synchronize()
    assert rel(Aq.cpu().numpy(), ref) < 1e-12


def test_fp64_split_large_and_scaled_inputs(nb, O, dev):
    """Double-float arithmetic keeps 1e-12 at a larger size and for inputs scaled
    over many orders of magnitude (ggeo ~1e-6, q ~1e5)."""
    N = 7
    m = O.BoxMesh(N, 6, 5, 4, perturb=0.1, seed=77)
    E, L = m.E, m.Nlocal
    lam, q = fields(O, L, 1, 78)
    for gs, qs in ((1.0, 1.0), (1e-6, 1e5), (1e3, 1e-7)):
        g, qq = m.ggeo * gs, q * qs
        for flags in (0, 1):
            ref = O.axhelm(N + 1, E, L, flags, g, m.D, lam, qq)
            Aq = torch.zeros(L, dtype=torch.float64, device=dev)
            nb.axhelm(N + 1, flags, nb.FP64_SPLIT, E, L, T(g, dev), T(m.D, dev), T(lam, dev),
                      T(qq, dev), Aq)
            torch.cuda.synchronize()
            assert rel(Aq.cpu().numpy(), ref) < 1e-12, (gs, qs, flags)


@pytest.mark.parametrize("name", ["axhelm_v0", "axhelm_bk_v0", "axhelm_n3_v0", "axhelm_bk_n3_v0"])
def test_reference_kernel_names(nb, O, dev, name):
    N = 7
    m = O.BoxMesh(N, 4, 3, 2, perturb=0.1, seed=5)
    k = nb.load_ax_kernel(name, N)
    E, L = m.E, m.Nlocal
    nf = 3 if "n3" in name else 1
    lam, q = fields(O, L, nf, 7)
    Aq = torch.zeros(nf * L, dtype=torch.float64, device=dev)
    k(E, L, T(m.ggeo, dev), T(m.D, dev), T(lam, dev), T(q, dev), Aq)
    torch.cuda.synchronize()
    ref = O.axhelm(N + 1, E, L, k.flags, m.ggeo, m.D, lam, q)
    assert rel(Aq.cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize("name", ["axhelmPartial_v0", "axhelmPartial_bk_n3_v0"])
def test_partial_element_list(nb, O, dev, name):
    N = 5
    m = O.BoxMesh(N, 3, 3, 2, perturb=0.1, seed=9)
    E, L = m.E, m.Nlocal
    k = nb.load_ax_kernel(name, N)
    nf = 3 if k.flags & nb.AX_N3 else 1
    lam, q = fields(O, L, nf, 11)
    rng = np.random.default_rng(0)
    elist = np.sort(rng.choice(E, size=E // 2, replace=False)).astype(np.int32)
    sentinel = 12345.0
    Aq = torch.full((nf * L,), sentinel, dtype=torch.float64, device=dev)
    k(len(elist), L, T(elist, dev), T(m.ggeo, dev), T(m.D, dev), T(lam, dev), T(q, dev), Aq)
    torch.cuda.synchronize()
    ref = np.full(nf * L, sentinel)
    O.axhelm(N + 1, len(elist), L, k.flags, m.ggeo, m.D, lam, q, element_list=elist, out=ref)
    got = Aq.cpu().numpy()
    assert rel(got, ref) < 1e-12
    # elements not in the list are untouched
    Np = m.Np
    untouched = np.setdiff1d(np.arange(E), elist)
    for f in range(nf):
        for e in untouched:
            assert np.all(got[f * L + e * Np: f * L + (e + 1) * Np] == sentinel)


def test_reference_driver_inputs(nb, O, dev):
    """The axhelm driver's own inputs: Gauss-node D, U[0,1) ggeo and q, lambda1=1.1."""
    N, E = 7, 37
    Nq, Np = N + 1, (N + 1) ** 3
    r, _ = O.gauss(N)
    D = O.dmatrix(r)
    ggeo = O.uniform(7 * Np * E, 42, 1, 0, 1)
    q = O.uniform(Np * E, 42, 2, 0, 1)
    lam = np.concatenate([np.ones(Np * E), 1.1 * np.ones(Np * E)])
    for flags in (0, 1):
        ref = O.axhelm(Nq, E, Np * E, flags, ggeo, D, lam, q)
        Aq = torch.zeros(Np * E, dtype=torch.float64, device=dev)
        nb.axhelm(Nq, flags, nb.FP64, E, Np * E, T(ggeo, dev), T(D, dev), T(lam, dev), T(q, dev), Aq)
        torch.cuda.synchronize()
        assert rel(Aq.cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize("N", [3, 7, 8, 9, 10, 11])
@pytest.mark.parametrize("flags", [0, 1, 2])
def test_fp32(nb, O, dev, N, flags):
    m = O.BoxMesh(N, 3, 3, 2, perturb=0.1, seed=21)
    E, L = m.E, m.Nlocal
    nf = 3 if flags & nb.AX_N3 else 1
    lam, q = fields(O, L, nf, 23)
    g32, D32, l32, q32 = (np.asarray(a, np.float32) for a in (m.ggeo, m.D, lam, q))
    ref = O.axhelm(N + 1, E, L, flags, g32.astype(np.float64), D32.astype(np.float64),
                   l32.astype(np.float64), q32.astype(np.float64))
    Aq = torch.zeros(nf * L, dtype=torch.float32, device=dev)
    nb.axhelm(N + 1, flags, nb.FP32, E, L, T(g32, dev), T(D32, dev), T(l32, dev), T(q32, dev), Aq)
    torch.cuda.synchronize()
    assert rel(Aq.cpu().numpy().astype(np.float64), ref) < 2e-5


@pytest.mark.parametrize("N", [7, 9])
@pytest.mark.parametrize("flags", [0, 1, 2])
def test_bf16_storage(nb, O, dev, N, flags):
    m = O.BoxMesh(N, 3, 2, 2, perturb=0.1, seed=31)
    E, L = m.E, m.Nlocal
    nf = 3 if flags & nb.AX_N3 else 1
    lam, q = fields(O, L, nf, 33)
    gb, lb = bf16_round(m.ggeo), bf16_round(lam)
    D32, q32 = np.asarray(m.D, np.float32), np.asarray(q, np.float32)
    ref = O.axhelm(N + 1, E, L, flags, gb, D32.astype(np.float64), lb, q32.astype(np.float64))
    Aq = torch.zeros(nf * L, dtype=torch.float32, device=dev)
    g_dev = T(m.ggeo, dev).to(torch.float32).to(torch.bfloat16)
    l_dev = T(lam, dev).to(torch.float32).to(torch.bfloat16)
    assert np.array_equal(g_dev.to(torch.float64).cpu().numpy(), gb)
    nb.axhelm(N + 1, flags, nb.BF16, E, L, g_dev, T(D32, dev), l_dev, T(q32, dev), Aq)
    torch.cuda.synchronize()
    assert rel(Aq.cpu().numpy().astype(np.float64), ref) < 2e-5
    # and against the unrounded FP64 operator: the storage error the solver sees
    ref64 = O.axhelm(N + 1, E, L, flags, m.ggeo, m.D, lam, q)
    assert rel(Aq.cpu().numpy().astype(np.float64), ref64) < 2e-2


@pytest.mark.parametrize("N", [2, 7, 9])
@pytest.mark.parametrize("flags", [0, 1, 2])
def test_trilinear_geometry(nb, O, dev, N, flags):
    m = O.BoxMesh(N, 3, 2, 3, perturb=0.1, seed=41)
    E, L = m.E, m.Nlocal
    nf = 3 if flags & nb.AX_N3 else 1
    lam, q = fields(O, L, nf, 43)
    ref = O.axhelm(N + 1, E, L, flags, m.ggeo, m.D, lam, q)
    coef = torch.zeros(24 * E, dtype=torch.float32, device=dev)
    nb.trilinear_coeffs(E, T(m.EX, dev), T(m.EY, dev), T(m.EZ, dev), coef)
    Aq = torch.zeros(nf * L, dtype=torch.float32, device=dev)
    nb.axhelm(N + 1, flags, nb.FP32_TRILINEAR, E, L, coef, T(m.D, dev, torch.float32),
              T(lam, dev, torch.float32), T(q, dev, torch.float32), Aq)
    torch.cuda.synchronize()
    assert rel(Aq.cpu().numpy().astype(np.float64), ref) < 1e-5


def test_edge_cases(nb, O, dev):
    N = 7
    m = O.BoxMesh(N, 1, 1, 1, perturb=0.0, seed=1)  # a single element
    L = m.Nlocal
    lam, q = fields(O, L, 1, 3)
    ref = O.axhelm(N + 1, 1, L, 0, m.ggeo, m.D, lam, q)
    Aq = torch.zeros(L, dtype=torch.float64, device=dev)
    nb.axhelm(N + 1, 0, nb.FP64, 1, L, T(m.ggeo, dev), T(m.D, dev), T(lam, dev), T(q, dev), Aq)
    torch.cuda.synchronize()
    assert rel(Aq.cpu().numpy(), ref) < 1e-12
    # zero elements: no work, no error
    nb.axhelm(N + 1, 0, nb.FP64, 0, 0, T(m.ggeo, dev), T(m.D, dev), T(lam, dev), T(q, dev), Aq)
    # constant field in the kernel of the Laplacian (BK): A*1 = 0
    ones = torch.ones(L, dtype=torch.float64, device=dev)
    nb.axhelm(N + 1, nb.AX_BK, nb.FP64, 1, L, T(m.ggeo, dev), T(m.D, dev), None, ones, Aq)
    torch.cuda.synchronize()
    assert float(Aq.abs().max()) < 1e-12
    # argument errors come back as status codes
    with pytest.raises(nb.NekbError):
        nb.axhelm(13, 0, nb.FP64, 1, L, T(m.ggeo, dev), T(m.D, dev), T(lam, dev), T(q, dev), Aq)
    with pytest.raises(nb.NekbError):
        nb.axhelm(N + 1, 0, nb.FP64, 1, L, T(m.ggeo, dev), T(m.D, dev), None, T(q, dev), Aq)
    with pytest.raises(nb.NekbError):
        nb.axhelm(N + 1, nb.AX_PARTIAL, nb.FP64, 1, L, T(m.ggeo, dev), T(m.D, dev), T(lam, dev),
                  T(q, dev), Aq)


def test_symmetry_and_linearity(nb, O, dev):
    """Size-independent properties at a larger size: (u, A v) = (A u, v) and linearity."""
    N = 7
    bp = nb.BP(N, 12, 12, 12, perturb=0.1, seed=3)
    L = bp.Nlocal
    ggeo = bp.device_array("ggeo", 7 * L, torch.float64)
    D = bp.device_array("D", (N + 1) ** 2, torch.float64)
    g = torch.Generator(device="cpu").manual_seed(0)
    u = torch.rand(L, generator=g, dtype=torch.float64).to(dev)
    v = torch.rand(L, generator=g, dtype=torch.float64).to(dev)
    lam = torch.cat([torch.rand(L, generator=g, dtype=torch.float64) + 0.5,
                     torch.rand(L, generator=g, dtype=torch.float64) + 0.5]).to(dev)
    Au, Av, Auv = (torch.zeros(L, dtype=torch.float64, device=dev) for _ in range(3))
    for src, dst in ((u, Au), (v, Av), (2.0 * u - 3.0 * v, Auv)):
        nb.axhelm(N + 1, 0, nb.FP64, bp.E, L, ggeo, D, lam, src, dst)
    torch.cuda.synchronize()
    s1, s2 = float(torch.dot(u, Av)), float(torch.dot(Au, v))
    assert abs(s1 - s2) / abs(s1) < 1e-12
    lin = (Auv - (2.0 * Au - 3.0 * Av)).abs().max() / Auv.abs().max()
    assert float(lin) < 1e-12


@pytest.mark.parametrize("N,ndim,bk", [(3, 1, True), (7, 3, False), (9, 1, False)])
def test_axhelm_driver(N, ndim, bk):
    """The axhelm driver on the reference driver's inputs (Gauss D, random
    ggeo and q): figures reported, double-float within 1e-12 and FP32 within
    1e-5 (relative, max-norm) of the FP64 kernel."""
    from nekbench_gb300 import axhelm_driver as drv
    base = ["--N", str(N), "--E", "512", "--ndim", str(ndim), "--steps", "3", "--json"]
    if bk:
        base.append("--bk")
    r64 = drv.main(base)
    assert r64["gdofs"] > 0 and r64["gbs"] > 0 and r64["gflops"] > 0
    rs = drv.main(base + ["--precision", "fp64_split"])
    assert rs["max_rel_diff_to_fp64"] < 1e-12
    r32 = drv.main(base + ["--precision", "fp32"])
    assert r32["max_rel_diff_to_fp64"] < 1e-5


def test_config1_e512_against_axhelm_reference(nb, O, dev):
    """The first configuration at its stated size: FP64 Poisson (BK), N=7,
    E=8x8x8=512 elements of the perturbed unit box (262,144 local nodes),
    q ~ U[-1,1].  Compared with axhelmReference.cpp's output (the fixture
    tests/golden/axhelm_config1_e512.npz: 4298 sampled nodes plus the whole
    array's sum, sum of squares and max-abs) and, at every node, with the
    oracle; 1e-12 relative (max-norm), the FP64 bar."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "axhelm_config1_e512.npz"))
    N, n, seed = int(g["N"]), int(g["n"]), int(g["seed"])
    m = O.BoxMesh(N, n, n, n, perturb=0.1, seed=seed)
    E, L = m.E, m.Nlocal
    assert E == 512 and L == 262144
    q = O.uniform(L, seed, 3, -1.0, 1.0)
    idx = g["idx"]
    assert rel(m.ggeo[idx], g["ggeo_samples"]) < 1e-14 and np.array_equal(q[idx], g["q_samples"])
    for name in ("axhelm_bk_v0",):
        k = nb.load_ax_kernel(name, N)
        Aq = torch.zeros(L, dtype=torch.float64, device=dev)
        k(E, L, T(m.ggeo, dev), T(m.D, dev), torch.zeros(2 * L, dtype=torch.float64, device=dev),
          T(q, dev), Aq)
        torch.cuda.synchronize()
        got = Aq.cpu().numpy()
        scale = float(g["Aq_maxabs"])
        assert np.abs(got[idx] - g["Aq_samples"]).max() / scale < 1e-12
        assert abs(np.abs(got).max() - scale) / scale < 1e-12
        assert abs((got * got).sum() - float(g["Aq_sumsq"])) / float(g["Aq_sumsq"]) < 1e-12
        ref = O.axhelm(N + 1, E, L, nb.AX_BK, m.ggeo, m.D, np.zeros(2 * L), q)
        assert rel(got, ref) < 1e-12


@pytest.mark.parametrize("prec", ["FP64", "FP64_SPLIT"])
@pytest.mark.parametrize("N", [5, 7, 8])
@pytest.mark.parametrize("flags", [0, 1, 2, 7])
def test_fp64_any_derivative_matrix(nb, O, dev, N, flags, prec):
    """The FP64 and double-float kernels evaluate the even-odd form only for a
    centro-antisymmetric D (nodes symmetric about the element centre); for any
    other D they must evaluate the direct sums.  A random D, and a GLL D with
    one entry moved by 1e-9, against the oracle at 1e-12 (the double-float
    precision has no Partial forms)."""
    if prec == "FP64_SPLIT" and flags & nb.AX_PARTIAL:
        pytest.skip("Partial variants run in FP64")
    m = O.BoxMesh(N, 3, 2, 2, perturb=0.1, seed=60 + N)
    E, L = m.E, m.Nlocal
    nf = 3 if flags & nb.AX_N3 else 1
    lam, q = fields(O, L, nf, 61 + N)
    Drand = O.uniform((N + 1) ** 2, 62, N, -2, 2)
    Dnudge = m.D.copy()
    Dnudge[1] += 1e-9
    for D in (Drand, Dnudge, m.D):
        if flags & nb.AX_PARTIAL:
            elist = np.arange(E - 1, -1, -2, dtype=np.int32)
            ref = np.full(nf * L, 3.0)
            O.axhelm(N + 1, len(elist), L, flags, m.ggeo, D, lam, q, element_list=elist, out=ref)
            Aq = torch.full((nf * L,), 3.0, dtype=torch.float64, device=dev)
            nb.axhelm(N + 1, flags, nb.FP64, len(elist), L, T(m.ggeo, dev), T(D, dev), T(lam, dev),
                      T(q, dev), Aq, element_list=T(elist, dev))
        else:
            ref = O.axhelm(N + 1, E, L, flags, m.ggeo, D, lam, q)
            Aq = torch.zeros(nf * L, dtype=torch.float64, device=dev)
            nb.axhelm(N + 1, flags, getattr(nb, prec), E, L, T(m.ggeo, dev), T(D, dev), T(lam, dev),
                      T(q, dev), Aq)
        torch.cuda.synchronize()
        assert rel(Aq.cpu().numpy(), ref) < 1e-12


def test_overlap_form_of_the_operator(nb, dev):
    """BPAxOperator's overlap form (nekBone/solve.cpp:189-211): the operator on
    the elements whose nodes other ranks share, the gather-scatter started, the
    operator on the other elements, the gather-scatter finished.  On one GPU it
    is composed from the Partial operator over the two element lists and one
    gather-scatter after both; for any partition of the elements the result is
    the plain operator followed by the gather-scatter, bit for bit."""
    N = 7
    bp = nb.BP(N, 4, 3, 3, perturb=0.1, seed=11)
    E, L = bp.E, bp.Nlocal
    ggeo = bp.device_array("ggeo", 7 * L, torch.float64)
    D = bp.device_array("D", (N + 1) ** 2, torch.float64)
    g = torch.Generator(device="cpu").manual_seed(5)
    q = torch.rand(L, generator=g, dtype=torch.float64).to(dev)
    lam = (torch.rand(2 * L, generator=g, dtype=torch.float64) + 0.5).to(dev)
    every = np.arange(E, dtype=np.int32)
    halo = torch.from_numpy(every[every % 3 == 0].copy()).to(dev)
    interior = torch.from_numpy(every[every % 3 != 0].copy()).to(dev)
    for flags in (0, nb.AX_BK):
        full = torch.zeros(L, dtype=torch.float64, device=dev)
        nb.axhelm(N + 1, flags, nb.FP64, E, L, ggeo, D, lam, q, full)
        bp.ogs.gather_scatter_many(full)
        split = torch.zeros(L, dtype=torch.float64, device=dev)
        for part in (halo, interior):
            nb.axhelm(N + 1, flags | nb.AX_PARTIAL, nb.FP64, len(part), L, ggeo, D, lam, q, split,
                      element_list=part)
        bp.ogs.gather_scatter_many(split)
        torch.cuda.synchronize()
        assert torch.equal(split, full), flags
