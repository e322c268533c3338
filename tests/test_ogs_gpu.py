"""Gather-scatter on the GPU: the CSR setup is bit-exact against the oracle's
restatement of ogsSetup (3rdParty/ogs/src/ogsSetup.cpp:137-212, 325-352) and
the sums are bit-exact against gatherScatterMany_doubleAdd's CSR order
(3rdParty/ogs/okl/gatherScatterMany.okl:58-85)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def T(x, dev):
    return torch.from_numpy(np.ascontiguousarray(x)).to(dev)


def assert_same_setup(nb, O, ids):
    g = nb.ogs_setup(ids)
    Ng, offs, gids, invdeg = O.ogs_setup(ids)
    assert g.NlocalGather == Ng
    o2, i2 = g.csr()
    assert np.array_equal(o2, offs)
    assert np.array_equal(i2, gids)
    assert np.array_equal(g.inv_degree().cpu().numpy(), invdeg)
    return g, (Ng, offs, gids, invdeg)


@pytest.mark.parametrize("periodic,dirichlet", [(False, True), (True, False), (False, False)])
@pytest.mark.parametrize("N", [1, 3, 7])
def test_box_setup_bit_exact(nb, O, N, periodic, dirichlet):
    m = O.BoxMesh(N, 3, 2, 4, periodic=periodic, dirichlet=dirichlet)
    assert_same_setup(nb, O, m.ids)


def test_random_ids_with_collisions_and_zeros(nb, O):
    rng = np.random.default_rng(5)
    for n, hi in ((1, 3), (17, 4), (1000, 50), (5000, 4000), (3000, 10**12)):
        ids = rng.integers(0, hi, size=n).astype(np.int64)
        ids[rng.random(n) < 0.1] = 0
        assert_same_setup(nb, O, ids)


def test_signed_ids(nb, O):
    """ogsSetup.cpp:161-166 opens a gather node at every change of the signed
    id in (|id|, local index) order: 5, -5, 5 are three groups, not one."""
    g, (Ng, _, _, _) = assert_same_setup(nb, O, np.array([5, -5, 5], dtype=np.int64))
    assert Ng == 3 and g.Nmulti == 0
    g, (Ng, offs, gids, _) = assert_same_setup(nb, O, np.array([5, 5, -5, 0, -5], dtype=np.int64))
    assert Ng == 2 and list(gids) == [0, 1, 2, 4]
    rng = np.random.default_rng(6)
    for n, hi in ((17, 4), (1000, 50), (5000, 4000), (3000, 10**12), (200000, 30000)):
        ids = rng.integers(0, hi, size=n).astype(np.int64)
        ids[rng.random(n) < 0.3] *= -1
        ids[rng.random(n) < 0.1] = 0
        assert_same_setup(nb, O, ids)


def test_signed_ids_gs_sums(nb, O, dev):
    rng = np.random.default_rng(8)
    ids = rng.integers(1, 700, size=20000).astype(np.int64)
    ids[rng.random(20000) < 0.5] *= -1
    g, (Ng, offs, gids, _) = assert_same_setup(nb, O, ids)
    v = O.uniform(len(ids), 4, 1, -1, 1)
    vd = T(v, dev)
    g.gather_scatter_many(vd)
    torch.cuda.synchronize()
    O.gs_many_add(Ng, offs, gids, v)
    assert np.array_equal(vd.cpu().numpy(), v)


def test_empty_and_all_zero(nb, O):
    g = nb.ogs_setup(np.zeros(10, dtype=np.int64))
    assert g.NlocalGather == 0 and g.Nlocal == 0
    assert np.array_equal(g.inv_degree().cpu().numpy(), np.ones(10))
    g = nb.ogs_setup(np.arange(1, 11, dtype=np.int64))  # all singletons
    assert g.NlocalGather == 10 and g.Nmulti == 0


@pytest.mark.parametrize("k", [1, 3])
def test_gs_many_double_bit_exact(nb, O, dev, k):
    m = O.BoxMesh(5, 4, 3, 3)
    L = m.Nlocal
    g, (Ng, offs, gids, _) = assert_same_setup(nb, O, m.ids)
    stride = L + 17  # stride larger than N, like fieldOffset with halo padding
    v = O.uniform(k * stride, 9, 1, -1, 1)
    vd = T(v, dev)
    g.gather_scatter_many(vd, k, stride, "double", "add")
    torch.cuda.synchronize()
    O.gs_many_add(Ng, offs, gids, v, k, stride)
    assert np.array_equal(vd.cpu().numpy(), v)


def test_gs_float(nb, O, dev):
    m = O.BoxMesh(7, 3, 3, 3)
    g, (Ng, offs, gids, _) = assert_same_setup(nb, O, m.ids)
    v = O.uniform(m.Nlocal, 2, 2, -1, 1).astype(np.float32)
    vd = T(v, dev)
    g.gather_scatter_many(vd, 1, 0, "float", "add")
    torch.cuda.synchronize()
    # float sums in the same order as a float32 restatement
    ref = v.copy()
    for q in range(Ng):
        s, e = offs[q], offs[q + 1]
        if e - s < 2:
            continue
        acc = np.float32(0)
        for n in gids[s:e]:
            acc = np.float32(acc + ref[n])
        ref[gids[s:e]] = acc
    assert np.array_equal(vd.cpu().numpy(), ref)


@pytest.mark.parametrize("periodic", [True, False])
def test_known_answer_gs_benchmark(nb, O, dev, periodic):
    """gs/main.cpp:136-193: sum(nearbyint(gs(1/gs(1)))) equals the number of local nodes."""
    m = O.BoxMesh(7, 4, 3, 2, periodic=periodic, dirichlet=not periodic)
    g = nb.ogs_setup(m.ids)
    q = torch.ones(m.Nlocal, dtype=torch.float64, device=dev)
    g.gather_scatter_many(q)
    q = 1.0 / q
    g.gather_scatter_many(q)
    torch.cuda.synchronize()
    assert int(torch.round(q).sum()) == m.Nlocal


def test_mask_kernel(nb, O, dev):
    m = O.BoxMesh(3, 2, 2, 2)
    q = torch.ones(m.Nlocal, dtype=torch.float64, device=dev)
    nb.mask(T(m.maskIds, dev), q)
    torch.cuda.synchronize()
    ref = np.ones(m.Nlocal)
    O.lib().nekbo_mask(len(m.maskIds), m.maskIds, ref)
    assert np.array_equal(q.cpu().numpy(), ref)


@pytest.mark.parametrize("N", list(range(1, 14)))
def test_update_jacobi_bit_exact(nb, O, dev, N):
    """nekb_update_jacobi against the oracle's statement of updateJacobi
    (nekBone/kernel/updateJacobi.okl:27-108), bit for bit: perturbed
    geometry, variable lambda0 and a nonzero lambda1, the Poisson case
    (lambda0 = 1, lambda1 = 0), with and without the boundary mask mapB."""
    m = O.BoxMesh(N, 3, 2, 2, perturb=0.1, seed=40 + N)
    E, L = m.E, m.Nlocal
    mapB = np.zeros(L, dtype=np.int32)
    mapB[m.maskIds] = 1
    lams = {"helmholtz": np.concatenate([O.uniform(L, N, 1, 0.5, 1.5), O.uniform(L, N, 2, 0.5, 2.0)]),
            "poisson": np.concatenate([np.ones(L), np.zeros(L)])}
    for lname, lam in lams.items():
        for mb in (None, mapB):
            ref = O.update_jacobi(N + 1, E, L, m.ggeo, m.D, lam, mb)
            diag = torch.full((L,), -7.0, dtype=torch.float64, device=dev)
            nb.update_jacobi(N + 1, E, L, None if mb is None else T(mb, dev), T(m.ggeo, dev),
                             T(m.D, dev), T(lam, dev), diag)
            torch.cuda.synchronize()
            got = diag.cpu().numpy()
            assert np.array_equal(got, ref), (lname, mb is None, np.abs(got - ref).max())
            if mb is not None:
                assert np.all(got[m.maskIds] == 1.0)
