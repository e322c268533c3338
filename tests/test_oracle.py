"""CPU tests of the oracle (no GPU): pinned to golden vectors produced by the
reference's own CPU code (tests/golden/make_golden.py) and, where oracle/_ref
was built here, to that code directly; plus the reference's known-answer
checks and properties of the basis, mesh, gather-scatter, PCG and network."""
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("case", ["axhelm_n3", "axhelm_n7", "axhelm_n9"])
def test_axhelm_matches_reference_golden(case):
    g = np.load(os.path.join(GOLD, case + ".npz"))
    N, E = int(g["N"]), int(g["E"])
    Nq = N + 1
    L = E * Nq ** 3
    for variant in range(4):
        nf = 3 if variant & 2 else 1
        got = O.axhelm(Nq, E, L, variant, g["ggeo"], g["D"], g["lam"], g["q"][: nf * L].copy())
        # same loop structure and operation order as kernel/CPU/axhelm.c: bit-identical
        assert np.array_equal(got, g[f"Aq_cpu_v{variant}"]), variant
    # axhelmReference.cpp uses a scalar lambda (lambda0 = 1)
    for lam1 in (0.0, 1.1):
        lam = np.concatenate([np.ones(L), lam1 * np.ones(L)])
        flags = O.AX_BK if lam1 == 0.0 else 0
        got = O.axhelm(Nq, E, L, flags, g["ggeo"], g["D"], lam, g["q"][:L].copy())
        assert rel(got, g[f"Aq_reference_lam{lam1}"]) < 1e-14


def config1_inputs(g):
    """Rebuild the E=512 (8x8x8, N=7) perturbed box and q of the config-1
    fixture from its seed; the fixture's samples confirm the rebuild."""
    N, n, seed = int(g["N"]), int(g["n"]), int(g["seed"])
    m = O.BoxMesh(N, n, n, n, perturb=0.1, seed=seed)
    q = O.uniform(m.Nlocal, seed, 3, -1.0, 1.0)
    idx = g["idx"]
    assert rel(m.ggeo[idx], g["ggeo_samples"]) < 1e-14
    assert np.array_equal(q[idx], g["q_samples"])
    return m, q


def test_axhelm_config1_size_against_reference():
    """axhelm FP64 Poisson, N=7, E=8^3=512 perturbed box: the oracle's BK
    operator against axhelmReference.cpp's output (lambda = 0) at 4298
    sampled nodes and the whole array's sum, sum of squares and max-abs."""
    g = np.load(os.path.join(GOLD, "axhelm_config1_e512.npz"))
    m, q = config1_inputs(g)
    got = O.axhelm(m.Nq, m.E, m.Nlocal, O.AX_BK, m.ggeo, m.D, np.zeros(2 * m.Nlocal), q)
    scale = float(g["Aq_maxabs"])
    assert np.abs(got[g["idx"]] - g["Aq_samples"]).max() / scale < 1e-13
    assert abs(np.abs(got).max() - scale) / scale < 1e-13
    assert abs((got * got).sum() - float(g["Aq_sumsq"])) / float(g["Aq_sumsq"]) < 1e-12
    assert abs(got.sum() - float(g["Aq_sum"])) / (scale * m.Nlocal) < 1e-13


def test_uniform_generator_golden():
    g = np.load(os.path.join(GOLD, "uniform.npz"))
    assert np.array_equal(O.uniform(16, 5, 2), g["u_seed5_stream2"])
    assert np.array_equal(O.uniform(16, 0, 0), g["u_seed0_stream0"])


def test_weighted_inner_product_golden():
    g = np.load(os.path.join(GOLD, "weighted_inner_product.npz"))
    w, a, b = g["w"], g["a"], g["b"]
    n = len(w)
    L = O.lib()
    L.nekbo_wdot.restype = __import__("ctypes").c_double
    ab = L.nekbo_wdot(n, 1, n, w.ctypes.data, a.ctypes.data, b.ctypes.data)
    aa = L.nekbo_wdot(n, 1, n, w.ctypes.data, a.ctypes.data, a.ctypes.data)
    # weightedInnerProductUpdate (CPU/weightedInnerProduct.c:64): [sum w a b, sum w a a]
    assert rel(np.array([ab, aa]), g["wab"]) < 1e-13


@pytest.mark.parametrize("N", [7, 9, 3])
def test_live_reference_when_built(N):
    R = O.ref(N + 1)
    if R is None:
        pytest.skip("oracle/_ref not built (reference sources absent)")
    m = O.BoxMesh(N, 3, 2, 2, perturb=0.1, seed=N)
    E, L = m.E, m.Nlocal
    lam = np.concatenate([O.uniform(L, 1, 1, 0.5, 1.5), O.uniform(L, 1, 2, 0.5, 2.0)])
    q = O.uniform(3 * L, 1, 3, -1, 1)
    for variant in range(4):
        nf = 3 if variant & 2 else 1
        ref = np.zeros(nf * L)
        R.nekref_axhelm_cpu(variant, E, L, m.ggeo, m.D, lam.ctypes.data, q[: nf * L].copy(), ref)
        got = O.axhelm(N + 1, E, L, variant, m.ggeo, m.D, lam, q[: nf * L].copy())
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("N", range(1, 12))
def test_gll_basis(N):
    x, w = O.gll(N)
    assert x[0] == -1 and x[-1] == 1 and np.all(np.diff(x) > 0)
    assert np.array_equal(x, -x[::-1])
    D = O.dmatrix(x).reshape(N + 1, N + 1)
    for p in range(N + 1):  # D differentiates polynomials of degree <= N exactly
        f, df = x ** p, (p * x ** (p - 1) if p else 0 * x)
        assert np.abs(D @ f - df).max() < 1e-11 * (1 + np.abs(df).max())
    for p in range(2 * N):  # GLL quadrature is exact to degree 2N-1
        exact = (1 - (-1) ** (p + 1)) / (p + 1)
        assert abs(np.dot(w, x ** p) - exact) < 1e-13
    # centro-antisymmetry of D on symmetric nodes
    assert np.abs(D + D[::-1, ::-1]).max() < 1e-12


@pytest.mark.parametrize("N", [0, 1, 4, 7, 9])
def test_gauss_basis(N):
    x, w = O.gauss(N)
    for p in range(2 * N + 2):
        exact = (1 - (-1) ** (p + 1)) / (p + 1)
        assert abs(np.dot(w, x ** p) - exact) < 1e-13


def test_affine_box_geometric_factors():
    """Unperturbed box: G = JW*diag(1/hr^2), G01=G02=G12=0, JW = J w_i w_j w_k."""
    N, nx, ny, nz = 4, 2, 3, 5
    m = O.BoxMesh(N, nx, ny, nz, perturb=0.0)
    Np = m.Np
    x, w = O.gll(N)
    W = np.einsum("k,j,i->kji", w, w, w).ravel()
    hx, hy, hz = 1 / nx / 2, 1 / ny / 2, 1 / nz / 2  # d x / d r
    J = hx * hy * hz
    g = m.ggeo.reshape(m.E, 7, Np)
    assert np.abs(g[:, 0] - J * W).max() < 1e-15
    assert np.abs(g[:, 1] - J * W / hx ** 2).max() < 1e-12
    assert np.abs(g[:, 4] - J * W / hy ** 2).max() < 1e-12
    assert np.abs(g[:, 6] - J * W / hz ** 2).max() < 1e-12
    assert np.abs(g[:, [2, 3, 5]]).max() < 1e-13


def test_perturbed_mesh_is_valid_and_watertight():
    m = O.BoxMesh(7, 4, 4, 4, perturb=0.1, seed=2)
    assert np.all(m.ggeo.reshape(m.E, 7, m.Np)[:, 0] > 0)  # positive Jacobian
    # coincident nodes (same global id) have the same coordinates
    ids = m.ids
    nz = ids > 0
    order = np.argsort(ids[nz], kind="stable")
    xs = np.stack([m.x[nz], m.y[nz], m.z[nz]], 1)[order]
    same = np.diff(ids[nz][order]) == 0
    assert np.abs(xs[1:][same] - xs[:-1][same]).max() < 1e-14


@pytest.mark.parametrize("periodic", [False, True])
def test_ogs_known_answer(periodic):
    """gs/main.cpp:136-193: sum(nearbyint(gs(1/gs(1)))) == number of nodes."""
    m = O.BoxMesh(5, 3, 3, 2, periodic=periodic, dirichlet=not periodic)
    Ng, offs, gids, invdeg = O.ogs_setup(m.ids)
    q = np.ones(m.Nlocal)
    O.gs_many_add(Ng, offs, gids, q)
    q = 1 / q
    O.gs_many_add(Ng, offs, gids, q)
    assert int(np.rint(q).sum()) == m.Nlocal
    assert np.allclose(invdeg[m.ids > 0] * np.bincount(m.ids)[m.ids[m.ids > 0]], 1.0)


def test_ogs_csr_order():
    rng = np.random.default_rng(3)
    ids = rng.integers(0, 40, size=300).astype(np.int64)
    Ng, offs, gids, invdeg = O.ogs_setup(ids)
    nz = np.flatnonzero(ids)
    assert offs[-1] == len(nz) and sorted(gids) == list(nz)
    firsts = [gids[offs[g]] for g in range(Ng)]
    assert firsts == sorted(firsts)  # groups numbered by first local appearance
    for g in range(Ng):
        mem = gids[offs[g]:offs[g + 1]]
        assert np.all(np.diff(mem) > 0) and len(set(ids[mem])) == 1
        assert np.all(invdeg[mem] == 1.0 / len(mem))
    assert np.all(invdeg[ids == 0] == 1.0)


def ogs_setup_statement(ids):
    """Plain-Python statement of ogsSetup's local branch
    (3rdParty/ogs/src/ogsSetup.cpp:40-54, 137-212): order the nonzero ids by
    (|id|, local index), open a gather node at every change of the SIGNED id
    (:161-166), number the gather nodes by the local index of their first
    member (:173-189), list members in ascending local index (:197-205)."""
    nodes = sorted((abs(int(v)), i, int(v)) for i, v in enumerate(ids) if v != 0)
    groups = []
    for p, (_, lid, sid) in enumerate(nodes):
        if p == 0 or sid != nodes[p - 1][2]:
            groups.append([])
        groups[-1].append(lid)
    groups.sort(key=lambda g: g[0])
    offs = np.cumsum([0] + [len(g) for g in groups]).astype(np.int32)
    gids = np.array([n for g in groups for n in g], dtype=np.int32)
    invdeg = np.ones(len(ids))
    for g in groups:
        invdeg[g] = 1.0 / len(g)
    return len(groups), offs, gids, invdeg


@pytest.mark.parametrize("ids", [[5, -5, 5], [5, 5, -5], [-5, 5, 5], [-3, -3, 3, 0, 3, -3],
                                 [7, -7], [-7, -7], [0, 0, 0]])
def test_ogs_signed_ids_small(ids):
    ids = np.array(ids, dtype=np.int64)
    got = O.ogs_setup(ids)
    ref = ogs_setup_statement(ids)
    assert got[0] == ref[0]
    for a, b in zip(got[1:], ref[1:]):
        assert np.array_equal(a, b)
    if list(ids) == [5, -5, 5]:
        assert got[0] == 3  # one gather node per change of sign, as ogsSetup.cpp:163


def test_ogs_signed_ids_random():
    rng = np.random.default_rng(11)
    for n, hi in ((50, 5), (2000, 60), (3000, 10**12)):
        ids = rng.integers(0, hi, size=n).astype(np.int64)
        ids[rng.random(n) < 0.4] *= -1
        ids[rng.random(n) < 0.1] = 0
        got = O.ogs_setup(ids)
        ref = ogs_setup_statement(ids)
        assert got[0] == ref[0]
        for a, b in zip(got[1:], ref[1:]):
            assert np.array_equal(a, b)


def _problem(N=3, n=3, seed=4):
    m = O.BoxMesh(N, n, n, n, perturb=0.1, seed=seed)
    L = m.Nlocal
    lam = np.concatenate([O.uniform(L, seed, 1, 0.5, 1.5), O.uniform(L, seed, 2, 0.5, 2.0)])
    bp = O.BP(m, lam)
    f = O.uniform(L, seed, 3, -1, 1)
    O.gs_many_add(bp.Ng, bp.offs, bp.gids, f)
    O.lib().nekbo_mask(len(m.maskIds), m.maskIds, f)
    return m, bp, f


def test_assembled_operator_is_spd():
    m, bp, f = _problem()
    w = bp.invdeg
    u = O.uniform(m.Nlocal, 9, 1, -1, 1)
    v = O.uniform(m.Nlocal, 9, 2, -1, 1)
    for a in (u, v):
        O.gs_many_add(bp.Ng, bp.offs, bp.gids, a)
        a *= w  # continuous fields: average the element copies
        O.gs_many_add(bp.Ng, bp.offs, bp.gids, a)
        O.lib().nekbo_mask(len(m.maskIds), m.maskIds, a)
    Au, Av = bp.apply(u), bp.apply(v)
    s1, s2 = np.sum(w * u * Av), np.sum(w * Au * v)
    assert abs(s1 - s2) < 1e-12 * abs(s1)
    assert np.sum(w * u * Au) > 0


def test_pcg_converges_and_jacobi_helps():
    m, bp, f = _problem()
    x1, r1 = np.zeros_like(f), f.copy()
    it_j, hist = bp.pcg(r1, x1, 1e-8, 500, precond=1, hist=True)
    x0, r0 = np.zeros_like(f), f.copy()
    it_c = bp.pcg(r0, x0, 1e-8, 500, precond=0)
    assert 0 < it_j < it_c < 500
    assert hist[it_j] <= max(1e-16 * hist[0], 1e-16)
    res = f - bp.apply(x1)
    w = bp.invdeg
    assert np.sqrt(np.sum(w * res * res) / np.sum(w * f * f)) < 1.01e-8
    # flexible beta gives the same iterates for a fixed preconditioner
    x2, r2 = np.zeros_like(f), f.copy()
    it_f = bp.pcg(r2, x2, 1e-8, 500, precond=1, flexible=True)
    assert abs(it_f - it_j) <= 1 and rel(x2, x1) < 1e-6


_net_forward = O.net_forward
net_loss_grad = O.net_loss_grad


def test_network_gradient_by_finite_differences():
    Nq, C, E = 4, 4, 3
    P = 27 * C * (C + 2)
    rng = np.random.default_rng(1)
    W = (rng.standard_normal(P) * 0.3).astype(np.float32)
    x = rng.standard_normal(E * Nq ** 3).astype(np.float32)
    t = rng.standard_normal(E * Nq ** 3).astype(np.float32)
    loss, g = net_loss_grad(Nq, W, x, t, C)
    for p in rng.choice(P, 25, replace=False):
        h = 1e-2
        Wp, Wm = W.copy(), W.copy()
        Wp[p] += h
        Wm[p] -= h
        lp = np.mean((_net_forward(Nq, Wp, x, C)[0].astype(np.float64) - t) ** 2)
        lm = np.mean((_net_forward(Nq, Wm, x, C)[0].astype(np.float64) - t) ** 2)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[p]) < 2e-3 * (abs(fd) + 1e-2), (p, fd, g[p])


def test_gelu_oracle():
    x = np.linspace(-4, 4, 101).astype(np.float32)
    y = O.gelu(x)
    assert abs(y[50]) < 1e-7 and abs(y[-1] - 4 * 0.99993) < 1e-3
    gx = O.gelu_backward(x, np.ones_like(x))
    fd = (O.gelu(x + 1e-3) - O.gelu(x - 1e-3)) / 2e-3
    assert np.abs(gx - fd).max() < 5e-3


def _reference_mode_problem(nx, ny, nz):
    """nekBone BP mode (nekBone/setup.cpp:44-53, 76-98): periodic unperturbed box
    [-1,1]^3, N=7, Poisson (BK), rhs 3 pi^2 JW cos(pi x) cos(pi y) cos(pi z)
    assembled by gather-scatter, COPY preconditioner."""
    m = O.BoxMesh(7, nx, ny, nz, perturb=0.0, periodic=True, dirichlet=False, box=(-1.0, 1.0))
    L = m.E * m.Np
    JW = m.ggeo.reshape(m.E, 7, m.Np)[:, 0, :].reshape(-1)
    exact = np.cos(np.pi * m.x) * np.cos(np.pi * m.y) * np.cos(np.pi * m.z)
    bp = O.BP(m, np.concatenate([np.ones(L), np.zeros(L)]), bk=True)
    r = O.gs_many_add(bp.Ng, bp.offs, bp.gids, 3 * np.pi ** 2 * JW * exact)
    return m, bp, r, exact


def test_reference_mode_known_answer():
    """The reference's own correctness check (nekBone/main.cpp:105-131) on its
    BP5 case, N=7, E=16x16x32=8192, tol 1e-6: the published run reports
    maxError 1.02763e-07 in 78 iterations (nekBone/readme.md:39).  The oracle
    (solve() with BPZeroMean on r and x, nekBone/main.cpp:24-31) must take the
    same number of iterations and land within 3 % of that error."""
    m, bp, r, exact = _reference_mode_problem(16, 16, 32)
    L = m.E * m.Np
    O.zero_mean(r, L)
    x = np.zeros(L)
    it = bp.pcg(r, x, 1e-6, 1000, precond=0)
    O.zero_mean(x, L)
    err = np.abs(exact - x).max()
    assert it == 78
    assert abs(err - 1.02763e-07) <= 0.03 * 1.02763e-07


def test_zero_mean_restatement():
    q = O.uniform(3 * 40, 9, 1, -1, 1)
    q0 = q.copy()
    O.zero_mean(q, 30, Nfields=3, offset=40)  # 30 local nodes per field, stride 40
    mean = sum(q0[f * 40:f * 40 + 30].sum() for f in range(3)) / 90
    assert np.allclose(q, q0 - mean, rtol=0, atol=1e-15)


def test_openmp_pcg_baseline_matches_serial_oracle():
    """The CPU timing baseline (BPPCG on all host threads) converges like the
    ordered oracle PCG: same iteration count within 1, solution within 1e-8."""
    m = O.BoxMesh(5, 4, 4, 4, perturb=0.1, seed=5)
    L = m.Nlocal
    lam = np.concatenate([O.uniform(L, 5, 1, 0.5, 1.5), O.uniform(L, 5, 2, 0.5, 2.0)])
    bp = O.BP(m, lam)
    f = O.gs_many_add(bp.Ng, bp.offs, bp.gids, O.uniform(L, 5, 3, -1.0, 1.0))
    f[m.maskIds] = 0.0
    r1, x1 = f.copy(), np.zeros(L)
    it1 = bp.pcg(r1, x1, 1e-10, 1000)
    r2, x2 = f.copy(), np.zeros(L)
    it2, setup = bp.pcg_omp(r2, x2, 1e-10, 1000)
    assert abs(it1 - it2) <= 1 and it1 < 1000 and setup >= 0.0
    assert np.abs(x1 - x2).max() <= 1e-8 * np.abs(x1).max()


def test_bench_cpu_pcg_block_on_a_small_sample():
    import bench
    fake = {"fp64_jacobi": {"iterations": 100, "elapsed_s": 2.0}, "mixed_fp32": {"elapsed_s": 0.5}}
    out = bench.cpu_pcg_reference(fake, 8, seconds=0.05, n=2)
    assert out["kind"] == "port" and out["cores"] >= 1 and out["seconds_per_iteration"] > 0
    assert out["projected_time_to_1e-8_s"] == pytest.approx(
        out["seconds_per_iteration"] * (8 ** 3 / 2 ** 3) * 100)
    assert set(out["gpu_speedup"]) == {"fp64_jacobi", "mixed_fp32"}


@pytest.mark.parametrize("N", [1, 3, 7, 9, 13])
def test_cpu_baseline_port_matches_checker(N):
    """The timed CPU baseline (oracle/cpu_axhelm.c: the reference's CPU axhelm
    with the order fixed at compile time and multiply-add fusion allowed)
    agrees with the bit-identical checker to rounding, BK and Helmholtz; the
    OpenMP PCG that uses it takes the checker PCG's iteration count."""
    m = O.BoxMesh(N, 3, 2, 2, perturb=0.1, seed=70 + N)
    E, L = m.E, m.Nlocal
    q = O.uniform(L, N, 3, -1, 1)
    lam = np.concatenate([O.uniform(L, N, 1, 0.5, 1.5), O.uniform(L, N, 2, 0.5, 2.0)])
    for bk in (True, False):
        got = O.cpu_axhelm(N + 1, bk, E, L, m.ggeo, m.D, None if bk else lam, q, np.zeros(L))
        ref = O.axhelm(N + 1, E, L, O.AX_BK if bk else 0, m.ggeo, m.D, lam, q)
        assert rel(got, ref) < 1e-14
    if N == 7:
        bp = O.BP(m, lam)
        f = O.gs_many_add(bp.Ng, bp.offs, bp.gids, O.uniform(L, 5, 3, -1.0, 1.0))
        f[m.maskIds] = 0.0
        r1, x1, r2, x2 = f.copy(), np.zeros(L), f.copy(), np.zeros(L)
        it_omp, _ = bp.pcg_omp(r1, x1, 1e-8, 2000)
        it_chk = bp.pcg(r2, x2, 1e-8, 2000, precond=1)
        assert abs(it_omp - it_chk) <= 1 and rel(x1, x2) < 1e-7
