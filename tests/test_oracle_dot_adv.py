"""CPU checks of the oracle's dot and adv restatements (no GPU needed).

The dot and adv kernels of the reference exist only as OKL, compiled at run
time by the OCCA runtime, so the restatements cannot be pinned to reference
outputs here; they are checked against an independent numpy restatement and
against exact mathematical answers."""
import numpy as np
import pytest

import oracle as O
from adv_cases import einsum_adv, polynomial_case, random_case


def _tree(vals, B):
    """dot.okl:41-63 with numpy: halve each block in place, then s[0] + s[1]."""
    nb = -(-vals.size // B)
    s = np.zeros(nb * B)
    s[:vals.size] = vals
    s = s.reshape(nb, B)
    h = B // 2
    while h >= 2:
        s[:, :h] = s[:, :h] + s[:, h:2 * h]
        h //= 2
    return s[:, 0] + s[:, 1]


@pytest.mark.parametrize("B", [256, 512, 1024])
@pytest.mark.parametrize("N", [1, 255, 256, 257, 5000])
def test_dot_v0_tree(B, N):
    rng = np.random.default_rng(N + B)
    w, x, y = rng.random((3, N))
    p = O.dot_partials(0, w, x, y, block_size=B)
    assert np.array_equal(p, _tree(w * x * y, B))
    assert abs(p.sum() - np.dot(w * x, y)) < 1e-12 * N


def test_dot_v1_group_tree():
    """weightedInnerProduct2_v1 (dot.okl:114-169): groups of 32, then the 8 group sums."""
    rng = np.random.default_rng(3)
    N = 3 * 256 + 100
    w, x, y = rng.random((3, N))
    p = O.dot_partials(1, w, x, y)
    v = np.zeros(4 * 256)
    v[:N] = w * x * y
    g = _tree(v, 32).reshape(-1, 8)  # each group of 32 with the same halving steps
    for h in (4, 2, 1):
        g[:, :h] = g[:, :h] + g[:, h:2 * h]
    assert np.array_equal(p, g[:, 0])


def test_dot_block_fields():
    """weightedBlockInnerProduct2 (dot.okl:67-111): per node the sum over fields
    of w x y, w indexed per field like x and y."""
    rng = np.random.default_rng(4)
    N, off = 1000, 1024
    w, x, y = rng.random((3, 3 * off))
    p = O.dot_partials(2, w, x, y, N=N, Nfields=3, offset=off)
    per = np.zeros(N)
    for f in range(3):
        per = per + w[f * off:f * off + N] * x[f * off:f * off + N] * y[f * off:f * off + N]
    assert np.array_equal(p, _tree(per, 256))
    with pytest.raises(ValueError):
        O.dot_partials(2, w, x, y, N=N, Nfields=3, offset=N - 1)
    with pytest.raises(ValueError):
        O.dot_partials(1, w, x, y, N=N, block_size=512)


@pytest.mark.parametrize("N,cubN,gauss", [(3, 3, False), (7, 7, False), (4, 5, True),
                                          (7, 11, True), (9, 14, True)])
def test_adv_exact_polynomials(N, cubN, gauss):
    inp, exact = polynomial_case(N, cubN, 3, gauss)
    NU = O.adv_cubature(N + 1, cubN + 1, 3, **inp)
    assert np.abs(NU - exact).max() < 1e-12 * max(1.0, np.abs(exact).max())


@pytest.mark.parametrize("Nq,cubNq", [(3, 3), (4, 6), (8, 12)])
def test_adv_matches_einsum_restatement(Nq, cubNq):
    E = 3
    case = random_case(Nq, cubNq, E, seed=Nq)
    NU = O.adv_cubature(Nq, cubNq, E, **case)
    ref = einsum_adv(Nq, cubNq, E, **case)
    assert np.abs(NU - ref).max() <= 1e-13 * np.abs(ref).max()


def test_adv_is_quadratic_in_u_and_respects_offset():
    Nq, cq, E = 4, 6, 2
    case = random_case(Nq, cq, E, seed=7)
    NU = O.adv_cubature(Nq, cq, E, **case)
    c2 = dict(case, U=2.0 * case["U"])
    assert np.array_equal(O.adv_cubature(Nq, cq, E, **c2), 4.0 * NU)  # powers of two: exact
    Np, off = Nq ** 3, E * Nq ** 3 + 5
    U = np.zeros(3 * off)
    for f in range(3):
        U[f * off:f * off + E * Np] = case["U"][f * E * Np:(f + 1) * E * Np]
    NUo = O.adv_cubature(Nq, cq, E, **dict(case, U=U), offset=off)
    for f in range(3):
        assert np.array_equal(NUo[f * off:f * off + E * Np], NU[f * E * Np:(f + 1) * E * Np])


def test_dot_total_matches_the_compiled_reference_inner_product():
    """Summed in block order, the restated dot partials give the reference's
    own weighted inner product (nekBone/kernel/CPU/weightedInnerProduct.c:64,
    compiled unmodified into oracle/_ref) up to summation order: the same
    quantity, sum over nodes of w x y."""
    R = O.ref(8)
    if R is None:
        pytest.skip("reference CPU kernels not compiled here (oracle/Makefile target ref)")
    rng = np.random.default_rng(12)
    N = 300007
    w, x, y = rng.random((3, N))
    total = float(np.cumsum(O.dot_partials(0, w, x, y))[-1])
    wab = np.zeros(2)
    R.nekref_weighted_inner_product_update(N, N, w, x, y, wab)
    assert abs(total - wab[0]) <= 1e-13 * abs(wab[0])
