"""GPU parity of the dot benchmark kernels and the adv operator against the oracle.

dot: every per-block partial is bit-for-bit the oracle's (the kernels add in
the reference tree's order); adv: FP64 within 1e-12 of the largest |NU| (the
kernel contracts to FMAs, the oracle does not), exact polynomial answers, and
at full size the exact quadratic scaling NU(2u) = 4 NU(u)."""
import numpy as np
import pytest

from adv_cases import polynomial_case, random_case

pytestmark = pytest.mark.gpu

ADV_PAIRS = [(n, n) for n in range(2, 13)] + [(2, 3), (3, 5), (4, 6), (5, 8), (6, 9), (7, 11),
                                             (8, 12), (9, 14), (10, 15)]


def _dev(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("variant,B", [(0, 256), (0, 512), (0, 1024), (1, 256), (2, 256), (2, 1024)])
@pytest.mark.parametrize("N", [1, 255, 256, 257, 100003])
def test_dot_partials_bit_exact(nb, O, dev, variant, B, N):
    import torch
    rng = np.random.default_rng(N * 7 + B + variant)
    w, x, y = rng.random((3, N)) - 0.25
    ref = O.dot_partials(variant, w, x, y, block_size=B)
    out = torch.full((nb.dot_num_blocks(N, B),), np.nan, dtype=torch.float64, device=dev)
    assert out.numel() == ref.size
    nb.dot_partials(variant, N, _dev(w, dev), _dev(x, dev), _dev(y, dev), out, block_size=B)
    assert np.array_equal(out.cpu().numpy(), ref)


def test_dot_block_kernel_fields_and_api(nb, O, dev):
    import torch
    rng = np.random.default_rng(11)
    N, off = 70000, 70144
    w, x, y = rng.random((3, 3 * off))
    k = nb.load_dot_kernel("weightedBlockInnerProduct2", 512, Nfields=3)
    out = torch.zeros(nb.dot_num_blocks(N, 512), dtype=torch.float64, device=dev)
    k(N, off, _dev(w, dev), _dev(x, dev), _dev(y, dev), out)
    ref = O.dot_partials(2, w, x, y, N=N, Nfields=3, offset=off, block_size=512)
    assert np.array_equal(out.cpu().numpy(), ref)
    k0 = nb.load_dot_kernel("weightedInnerProduct2_v0")
    out0 = torch.zeros(nb.dot_num_blocks(N), dtype=torch.float64, device=dev)
    k0(N, _dev(w[:N], dev), _dev(x[:N], dev), _dev(y[:N], dev), out0)
    assert np.array_equal(out0.cpu().numpy(), O.dot_partials(0, w[:N], x[:N], y[:N]))
    # N = 0 writes nothing
    sentinel = torch.full((4,), 7.0, dtype=torch.float64, device=dev)
    nb.dot_partials(0, 0, sentinel, sentinel, sentinel, sentinel)
    assert torch.all(sentinel == 7.0)
    with pytest.raises(nb.NekbError):
        nb.dot_partials(1, N, out, out, out, out, block_size=512)
    with pytest.raises(nb.NekbError):
        nb.load_dot_kernel("weightedInnerProduct3_v0")


def test_dot_large_bit_exact(nb, O, dev):
    """2^25 + 7 nodes against the oracle."""
    import torch
    N = (1 << 25) + 7
    rng = np.random.default_rng(5)
    w, x, y = (rng.random(N) for _ in range(3))
    out = torch.empty(nb.dot_num_blocks(N), dtype=torch.float64, device=dev)
    nb.dot_partials(0, N, _dev(w, dev), _dev(x, dev), _dev(y, dev), out)
    assert np.array_equal(out.cpu().numpy(), O.dot_partials(0, w, x, y))


def test_dot_full_size_properties(nb, dev):
    """At the benchmark size (N=7, E=64^3: 134,217,728 nodes): swapping w and x
    and doubling w are exact operations on every partial."""
    import torch
    N = 512 * 64 ** 3
    g = torch.Generator(device=dev).manual_seed(3)
    w, x, y = (torch.rand(N, dtype=torch.float64, device=dev, generator=g) for _ in range(3))
    nblk = nb.dot_num_blocks(N)
    a, b, c = (torch.empty(nblk, dtype=torch.float64, device=dev) for _ in range(3))
    nb.dot_partials(0, N, w, x, y, a)
    nb.dot_partials(0, N, x, w, y, b)
    nb.dot_partials(0, N, 2 * w, x, y, c)
    torch.cuda.synchronize()
    assert torch.equal(a, b) and torch.equal(c, 2 * a)
    assert abs(a.sum().item() - torch.dot(w * x, y).item()) < 1e-9 * a.sum().item()


# tolerance relative to max |NU|: native FP64 (FMA contraction only) and
# double-float arithmetic (about 48 significant bits)
ADV_TOL = {0: 1e-12, 4: 1e-12}
ADV_POLY_TOL = {0: 1e-12, 4: 1e-10}


@pytest.mark.parametrize("precision", [0, 4], ids=["fp64", "fp64_split"])
@pytest.mark.parametrize("Nq,cubNq", ADV_PAIRS)
def test_adv_matches_oracle(nb, O, dev, Nq, cubNq, precision):
    import torch
    E = 5
    case = random_case(Nq, cubNq, E, seed=Nq * 31 + cubNq)
    ref = O.adv_cubature(Nq, cubNq, E, **case)
    d = {k: _dev(v, dev) for k, v in case.items()}
    NU = torch.full((3 * E * Nq ** 3,), np.nan, dtype=torch.float64, device=dev)
    nb.adv_cubature(Nq, cubNq, E, d["vgeo"], d["cubvgeo"], d["cubD"], d["cubInterpT"], E * Nq ** 3,
                    d["U"], NU, precision=precision)
    err = np.abs(NU.cpu().numpy() - ref).max()
    assert err <= ADV_TOL[precision] * np.abs(ref).max(), err


@pytest.mark.parametrize("precision", [0, 4], ids=["fp64", "fp64_split"])
@pytest.mark.parametrize("N,cubN,gauss", [(3, 3, False), (7, 7, False), (7, 11, True), (9, 14, True)])
def test_adv_exact_polynomials(nb, dev, N, cubN, gauss, precision):
    import torch
    E = 4
    inp, exact = polynomial_case(N, cubN, E, gauss)
    d = {k: _dev(v, dev) for k, v in inp.items()}
    NU = torch.empty(3 * E * (N + 1) ** 3, dtype=torch.float64, device=dev)
    k = nb.load_adv_kernel(N, cubN, precision)
    k(E, d["vgeo"], d["cubvgeo"], d["cubD"], d["cubInterpT"], E * (N + 1) ** 3, d["U"], NU)
    err = np.abs(NU.cpu().numpy() - exact).max()
    assert err < ADV_POLY_TOL[precision] * max(1.0, np.abs(exact).max()), err


@pytest.mark.parametrize("precision", [0, 4], ids=["fp64", "fp64_split"])
def test_adv_full_size_quadratic_and_offset(nb, dev, precision):
    """N=7, cubN=11 on 8192 elements (1.36 GB of cubature metric terms): doubling
    U multiplies NU by exactly 4 (every operation of both arithmetics scales
    exactly by powers of two); a padded field offset gives the same values."""
    import torch
    Nq, cq, E = 8, 12, 8192
    Np = Nq ** 3
    g = torch.Generator(device=dev).manual_seed(9)
    r = lambda n: torch.rand(n, dtype=torch.float64, device=dev, generator=g)  # noqa: E731
    vgeo, cub, D, I, U = r(12 * E * Np), r(12 * E * cq ** 3), r(cq * cq), r(Nq * cq), r(3 * E * Np)
    NU1, NU2 = (torch.empty(3 * E * Np, dtype=torch.float64, device=dev) for _ in range(2))
    nb.adv_cubature(Nq, cq, E, vgeo, cub, D, I, E * Np, U, NU1, precision)
    nb.adv_cubature(Nq, cq, E, vgeo, cub, D, I, E * Np, 2 * U, NU2, precision)
    torch.cuda.synchronize()
    assert torch.equal(NU2, 4 * NU1)
    off = E * Np + 64
    Up = torch.zeros(3 * off, dtype=torch.float64, device=dev)
    for f in range(3):
        Up[f * off:f * off + E * Np] = U[f * E * Np:(f + 1) * E * Np]
    NUp = torch.zeros(3 * off, dtype=torch.float64, device=dev)
    nb.adv_cubature(Nq, cq, E, vgeo, cub, D, I, off, Up, NUp, precision)
    for f in range(3):
        assert torch.equal(NUp[f * off:f * off + E * Np], NU1[f * E * Np:(f + 1) * E * Np])
    assert torch.all(NUp[E * Np:off] == 0)


def test_adv_errors(nb, dev):
    import torch
    t = torch.zeros(8, dtype=torch.float64, device=dev)
    with pytest.raises(nb.NekbError) as e:
        nb.adv_cubature(8, 13, 1, t, t, t, t, 512, t, t)
    assert e.value.code == nb.ERR_UNSUPPORTED
    with pytest.raises(nb.NekbError):
        nb.adv_cubature(8, 12, 2, t, t, t, t, 512, t, t)  # offset < E Np
    with pytest.raises(nb.NekbError) as e:
        nb.adv_cubature(8, 12, 1, t, t, t, t, 512, t, t, precision=nb.FP32)
    assert e.value.code == nb.ERR_UNSUPPORTED
    nb.adv_cubature(8, 12, 0, t, t, t, t, 0, t, t)      # no elements: nothing to do


def test_drivers(nb, dev):
    from nekbench_gb300 import adv, dot
    r = dot.main(["--E", "4096", "--steps", "3", "--json"])
    assert r["Nblock"] == (4096 * 512 + 255) // 256 and r["gbs"] > 0 and r["kernel_gbs"] > 0
    r = dot.main(["--E", "1000", "--steps", "2", "--kernel", "weightedBlockInnerProduct2",
                  "--block", "1024", "--json"])
    assert r["Nblock"] == 500
    r = adv.main(["--E", "256", "--steps", "2", "--json"])
    assert r["gdofs"] > 0 and r["flops_per_element"] == adv.flops(8, 12)
    r = adv.main(["--E", "256", "--steps", "2", "--precision", "fp64_split", "--json"])
    assert r["max_rel_diff_to_fp64"] < 1e-12
