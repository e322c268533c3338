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
