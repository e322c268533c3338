"""Inputs for the adv operator tests (numpy, float64).

``random_case`` fills every array as the reference driver does (uniform
random numbers, adv/main.cpp:98-103), here seeded.  ``polynomial_case`` builds
an identity-mapped element (x = r, y = s, z = t) whose advection term has an
exact answer: with the cubature on the GLL nodes, NU = (u . grad) u at the
nodes for any u of degree <= N; with Gauss cubature of order cubN >= 3N/2 - 1,
NU = (u . grad) u when that term has degree <= N - 1 per direction.
"""
import numpy as np

import oracle as O

# vgeo slots (core/params.h:2-13)
RX, RY, SX, SY, J, JW, IJW, RZ, SZ, TX, TY, TZ, NVGEO = range(13)


def lagrange(x, xc):
    """I[a, i] = l_a(xc_i): interpolation from nodes x to points xc."""
    n = len(x)
    I = np.ones((n, len(xc)))
    for a in range(n):
        for m in range(n):
            if m != a:
                I[a] *= (xc - x[m]) / (x[a] - x[m])
    return I


def random_case(Nq, cubNq, E, seed=1):
    rng = np.random.default_rng(seed)
    Np, cNp = Nq ** 3, cubNq ** 3
    return dict(vgeo=rng.random(E * Np * NVGEO), cubvgeo=rng.random(E * cNp * NVGEO),
                cubD=rng.random(cubNq * cubNq), cubInterpT=rng.random(Nq * cubNq),
                U=rng.random(3 * E * Np))


def polynomial_case(N, cubN, E, gauss):
    """Identity geometry and a velocity with a known advection term: returns
    (inputs, exact NU)."""
    Nq, cq = N + 1, cubN + 1
    r, w = O.gll(N)
    rc, wc = O.gauss(cubN) if gauss else (r, w)
    I = lagrange(r, rc)
    Np, cNp = Nq ** 3, cq ** 3
    vgeo = np.zeros((E, NVGEO, Np))
    cub = np.zeros((E, NVGEO, cNp))
    vgeo[:, IJW] = 1.0 / np.einsum("k,j,i->kji", w, w, w).ravel()
    cub[:, RX] = cub[:, SY] = cub[:, TZ] = 1.0
    cub[:, JW] = np.einsum("k,j,i->kji", wc, wc, wc).ravel()
    T, S, R = (a.ravel() for a in np.meshgrid(r, r, r, indexing="ij"))
    if gauss:  # (u . grad) u of degree 1
        u = [1 + R, 2 - S, 0.5 * T]
        f = [1 + R, S - 2, 0.25 * T]
    else:      # degree 3 (N >= 3)
        u = [R ** 2, S * T, np.ones_like(R)]
        f = [2 * R ** 3, S * T ** 2 + S, 0 * R]
    inputs = dict(vgeo=vgeo.ravel(), cubvgeo=cub.ravel(), cubD=O.dmatrix(rc).ravel(),
                  cubInterpT=I.ravel(), U=np.concatenate([np.tile(c, E) for c in u]))
    return inputs, np.concatenate([np.tile(c, E) for c in f])


def einsum_adv(Nq, cubNq, E, vgeo, cubvgeo, cubD, cubInterpT, U):
    """The same operator written with einsum (an independent restatement)."""
    I = cubInterpT.reshape(Nq, cubNq)           # [a, i]
    D = cubD.reshape(cubNq, cubNq)               # [i, n]
    u = U.reshape(3, E, Nq, Nq, Nq)              # [f, e, c, b, a]
    uc = np.einsum("ck,bj,ai,fecba->fekji", I, I, I, u)
    dr = np.einsum("in,fekjn->fekji", D, uc)
    ds = np.einsum("jn,fekni->fekji", D, uc)
    dt = np.einsum("kn,fenji->fekji", D, uc)
    g = cubvgeo.reshape(E, NVGEO, cubNq, cubNq, cubNq)
    hat = [g[:, JW] * (uc[0] * g[:, a] + uc[1] * g[:, b] + uc[2] * g[:, c])
           for a, b, c in ((RX, RY, RZ), (SX, SY, SZ), (TX, TY, TZ))]
    adv = hat[0] * dr + hat[1] * ds + hat[2] * dt
    nu = np.einsum("ck,bj,ai,fekji->fecba", I, I, I, adv)
    ijw = vgeo.reshape(E, NVGEO, Nq, Nq, Nq)[:, IJW]
    return (nu * ijw).ravel()
