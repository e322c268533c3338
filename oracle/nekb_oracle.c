/*
 * CPU oracle for the nekBench spectral-element hot path -- TEST INFRASTRUCTURE.
 *
 * Plain-C restatement of the reference algorithms (nekBench v20.0).  It is the
 * checker the GPU library is compared against; the library never links it and
 * never falls back to it.  Compile with -ffp-contract=off so that x86 and Arm
 * hosts produce identical bits.
 *
 * Pinned to the reference itself: the axhelm loops to its compiled CPU
 * kernels (kernel/CPU/axhelm.c, axhelmReference.cpp) and the weighted inner
 * product to kernel/CPU/weightedInnerProduct.c (tests/golden/make_golden.py);
 * gather-scatter, updateJacobi, the dot trees (v0, block) and adv at
 * cubNq = Nq to the reference's OKL kernels run with OCCA's Serial semantics
 * (oracle/okl_serial.py, tests/golden/make_okl_golden.py), bit for bit.
 */
#include "nekb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* counter-based random numbers: splitmix64 finaliser applied twice.          */
/* The library's device generator uses the same formula, so seeded inputs     */
/* are bit-identical on CPU and GPU.                                          */
/* ------------------------------------------------------------------------ */
static uint64_t mix64(uint64_t x)
{
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

uint64_t nekbo_hash(uint64_t seed, uint64_t stream, uint64_t i)
{
  return mix64(mix64(seed * 0xD1B54A32D192ED03ull + stream) + i);
}

double nekbo_uniform(uint64_t seed, uint64_t stream, uint64_t i)
{
  return (double)(nekbo_hash(seed, stream, i) >> 11) * (1.0 / 9007199254740992.0);
}

void nekbo_fill_uniform(double* v, int64_t n, uint64_t seed, uint64_t stream, double lo, double hi)
{
  const double span = hi - lo;
  for (int64_t i = 0; i < n; ++i) {
    double u = nekbo_uniform(seed, stream, (uint64_t)i);
    double t = span * u;
    v[i] = lo + t;
  }
}

/* ------------------------------------------------------------------------ */
/* 1D basis.  The reference builds GLL/Gauss nodes from the eigenvalues of   */
/* the Jacobi matrix (core/meshBasis.cpp:46-133, :140-173) and D by a        */
/* Vandermonde solve (:775-786).  Restated here with Newton iteration on the */
/* Legendre recurrences and the barycentric derivative formula, which give   */
/* the same nodes and matrix to rounding.                                    */
/* ------------------------------------------------------------------------ */
static void legendre(int n, double x, double* L, double* dL)
{
  /* L_n(x) and L_n'(x) by the three-term recurrence */
  double p0 = 1.0, p1 = x, d0 = 0.0, d1 = 1.0;
  if (n == 0) { *L = 1.0; *dL = 0.0; return; }
  for (int k = 2; k <= n; ++k) {
    double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    double d2 = d0 + (2.0 * k - 1.0) * p1;
    p0 = p1; p1 = p2; d0 = d1; d1 = d2;
  }
  *L = p1; *dL = d1;
}

int nekbo_gll(int N, double* x, double* w)
{
  const double pi = 3.14159265358979323846;
  if (N < 1) return -1;
  x[0] = -1.0; x[N] = 1.0;
  for (int j = 1; j <= N / 2; ++j) {
    /* interior nodes are the roots of L_N'(x): Newton on q = L_{N+1} - L_{N-1} */
    double xj = -cos(pi * j / N);
    for (int it = 0; it < 100; ++it) {
      double Lm, dLm, Lp, dLp;
      legendre(N - 1, xj, &Lm, &dLm);
      legendre(N + 1, xj, &Lp, &dLp);
      double q = Lp - Lm, dq = dLp - dLm;
      double delta = -q / dq;
      xj += delta;
      if (fabs(delta) <= 1e-16 * (1.0 + fabs(xj))) break;
    }
    x[j] = xj;
    x[N - j] = -xj;
  }
  if (N % 2 == 0) x[N / 2] = 0.0;
  for (int j = 0; j <= N; ++j) {
    double L, dL;
    legendre(N, x[j], &L, &dL);
    w[j] = 2.0 / (N * (N + 1.0) * L * L);
  }
  return N + 1;
}

int nekbo_gauss(int N, double* x, double* w)
{
  const double pi = 3.14159265358979323846;
  const int n = N + 1; /* roots of L_{N+1} */
  for (int j = 0; j < (n + 1) / 2; ++j) {
    double xj = -cos(pi * (2.0 * j + 1.0) / (2.0 * n));
    for (int it = 0; it < 100; ++it) {
      double L, dL;
      legendre(n, xj, &L, &dL);
      double delta = -L / dL;
      xj += delta;
      if (fabs(delta) <= 1e-16 * (1.0 + fabs(xj))) break;
    }
    x[j] = xj;
    x[n - 1 - j] = -xj;
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
  for (int j = 0; j < n; ++j) {
    double L, dL;
    legendre(n, x[j], &L, &dL);
    w[j] = 2.0 / ((1.0 - x[j] * x[j]) * dL * dL);
  }
  return n;
}

void nekbo_dmatrix(int Nq, const double* x, double* D)
{
  double* bw = (double*)malloc(sizeof(double) * Nq);
  for (int j = 0; j < Nq; ++j) {
    double p = 1.0;
    for (int k = 0; k < Nq; ++k)
      if (k != j) p *= (x[j] - x[k]);
    bw[j] = 1.0 / p;
  }
  for (int i = 0; i < Nq; ++i) {
    double diag = 0.0;
    for (int j = 0; j < Nq; ++j) {
      if (j == i) continue;
      double dij = (bw[j] / bw[i]) / (x[i] - x[j]);
      D[i * Nq + j] = dij;
      diag -= dij;
    }
    D[i * Nq + i] = diag;
  }
  free(bw);
}

/* ------------------------------------------------------------------------ */
/* box mesh                                                                  */
/* ------------------------------------------------------------------------ */
/* Element e = ex + nx*(ey + ny*ez); vertex order as core/meshSetup.cpp:2363-2410
 * (0:(i,j,k) 1:(i+1,j,k) 2:(i+1,j+1,k) 3:(i,j+1,k), 4..7 the same at k+1).
 * Box [box_min, box_max]^3 ([0,1]^3 when box_max <= box_min; the reference's
 * default is [-1,1]^3, core/meshSetup.cpp:2316-2353); interior vertices moved
 * by U[-perturb*h, perturb*h] per coordinate (random stream 1, counter
 * 3*vertex+c). */
void nekbo_box_vertices(int nx, int ny, int nz, double perturb, uint64_t seed, int periodic,
                        double box_min, double box_max, double* EX, double* EY, double* EZ)
{
  const int ext = box_max > box_min;
  const double lo = ext ? box_min : 0.0, len = ext ? box_max - box_min : 1.0;
  const double hx = len / nx, hy = len / ny, hz = len / nz;
  const int vi[8] = {0, 1, 1, 0, 0, 1, 1, 0};
  const int vj[8] = {0, 0, 1, 1, 0, 0, 1, 1};
  const int vk[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  for (int ez = 0; ez < nz; ++ez)
    for (int ey = 0; ey < ny; ++ey)
      for (int ex = 0; ex < nx; ++ex) {
        int64_t e = ex + (int64_t)nx * (ey + (int64_t)ny * ez);
        for (int v = 0; v < 8; ++v) {
          int I = ex + vi[v], J = ey + vj[v], K = ez + vk[v];
          double X = lo + I * hx, Y = lo + J * hy, Z = lo + K * hz;
          int interior = (I > 0 && I < nx && J > 0 && J < ny && K > 0 && K < nz);
          if (interior && !periodic && perturb != 0.0) {
            uint64_t vid = (uint64_t)I + (uint64_t)(nx + 1) * ((uint64_t)J + (uint64_t)(ny + 1) * K);
            double ux = nekbo_uniform(seed, 1, 3 * vid + 0);
            double uy = nekbo_uniform(seed, 1, 3 * vid + 1);
            double uz = nekbo_uniform(seed, 1, 3 * vid + 2);
            X += perturb * hx * (2.0 * ux - 1.0);
            Y += perturb * hy * (2.0 * uy - 1.0);
            Z += perturb * hz * (2.0 * uz - 1.0);
          }
          EX[e * 8 + v] = X; EY[e * 8 + v] = Y; EZ[e * 8 + v] = Z;
        }
      }
}

/* Global node numbering of the structured box: node (I,J,K) of the
 * (nx*N+1)x(ny*N+1)x(nz*N+1) lattice gets id 1+I+(nx*N+1)*(J+(ny*N+1)*K).
 * periodic: I is taken modulo nx*N (as the reference box, meshSetup.cpp:2363-2376).
 * dirichlet: nodes on the boundary get id 0, which excludes them from the
 * gather-scatter (ogs.hpp:42-44, ogsSetup.cpp:127,145). */
void nekbo_box_ids(int N, int nx, int ny, int nz, int periodic, int dirichlet, int64_t* ids)
{
  const int Nq = N + 1;
  const int64_t Np = (int64_t)Nq * Nq * Nq;
  const int64_t GX = (int64_t)nx * N + (periodic ? 0 : 1);
  const int64_t GY = (int64_t)ny * N + (periodic ? 0 : 1);
  for (int ez = 0; ez < nz; ++ez)
    for (int ey = 0; ey < ny; ++ey)
      for (int ex = 0; ex < nx; ++ex) {
        int64_t e = ex + (int64_t)nx * (ey + (int64_t)ny * ez);
        for (int k = 0; k < Nq; ++k)
          for (int j = 0; j < Nq; ++j)
            for (int i = 0; i < Nq; ++i) {
              int64_t I = (int64_t)ex * N + i, J = (int64_t)ey * N + j, K = (int64_t)ez * N + k;
              int64_t n = e * Np + i + Nq * (j + Nq * k);
              int bnd = (I == 0 || J == 0 || K == 0 || I == (int64_t)nx * N ||
                         J == (int64_t)ny * N || K == (int64_t)nz * N);
              if (periodic) {
                I %= (int64_t)nx * N; J %= (int64_t)ny * N; K %= (int64_t)nz * N;
                bnd = 0;
              }
              ids[n] = (dirichlet && bnd) ? 0 : 1 + I + GX * (J + GY * K);
            }
      }
}

int64_t nekbo_box_mask(int N, int nx, int ny, int nz, int32_t* maskIds)
{
  const int Nq = N + 1;
  const int64_t Np = (int64_t)Nq * Nq * Nq;
  int64_t cnt = 0;
  for (int ez = 0; ez < nz; ++ez)
    for (int ey = 0; ey < ny; ++ey)
      for (int ex = 0; ex < nx; ++ex) {
        int64_t e = ex + (int64_t)nx * (ey + (int64_t)ny * ez);
        for (int k = 0; k < Nq; ++k)
          for (int j = 0; j < Nq; ++j)
            for (int i = 0; i < Nq; ++i) {
              int64_t I = (int64_t)ex * N + i, J = (int64_t)ey * N + j, K = (int64_t)ez * N + k;
              int bnd = (I == 0 || J == 0 || K == 0 || I == (int64_t)nx * N ||
                         J == (int64_t)ny * N || K == (int64_t)nz * N);
              if (bnd) {
                if (maskIds) maskIds[cnt] = (int32_t)(e * Np + i + Nq * (j + Nq * k));
                cnt++;
              }
            }
      }
  return cnt;
}

/* trilinear map of the 8 vertices, restating meshPhysicalNodesHex3D (meshSetup.cpp:2156-2233) */
void nekbo_physical_nodes(int N, int64_t E, const double* r1d, const double* EX, const double* EY,
                          const double* EZ, double* x, double* y, double* z)
{
  const int Nq = N + 1;
  const int64_t Np = (int64_t)Nq * Nq * Nq;
  for (int64_t e = 0; e < E; ++e) {
    const double* xe = EX + 8 * e;
    const double* ye = EY + 8 * e;
    const double* ze = EZ + 8 * e;
    for (int k = 0; k < Nq; ++k)
      for (int j = 0; j < Nq; ++j)
        for (int i = 0; i < Nq; ++i) {
          double rn = r1d[i], sn = r1d[j], tn = r1d[k];
          double a[8] = {
            (1 - rn) * (1 - sn) * (1 - tn), (1 + rn) * (1 - sn) * (1 - tn),
            (1 + rn) * (1 + sn) * (1 - tn), (1 - rn) * (1 + sn) * (1 - tn),
            (1 - rn) * (1 - sn) * (1 + tn), (1 + rn) * (1 - sn) * (1 + tn),
            (1 + rn) * (1 + sn) * (1 + tn), (1 - rn) * (1 + sn) * (1 + tn)};
          double X = 0, Y = 0, Z = 0;
          for (int v = 0; v < 8; ++v) {
            X += 0.125 * a[v] * xe[v];
            Y += 0.125 * a[v] * ye[v];
            Z += 0.125 * a[v] * ze[v];
          }
          int64_t n = e * Np + i + Nq * (j + Nq * k);
          x[n] = X; y[n] = Y; z[n] = Z;
        }
  }
}

/* second-order geometric factors, restating meshGeometricFactorsHex3D
 * (meshSetup.cpp:255-360): derivatives of the nodal coordinates by D, the
 * inverse Jacobian, and G = JW * (grad r_a . grad r_b), slot order
 * GWJ,G00,G01,G02,G11,G12,G22 (core/params.h:55-62). */
void nekbo_geometric_factors(int N, int64_t E, const double* w1d, const double* D, const double* x,
                             const double* y, const double* z, double* ggeo)
{
  const int Nq = N + 1;
  const int64_t Np = (int64_t)Nq * Nq * Nq;
  for (int64_t e = 0; e < E; ++e) {
    const double* xe = x + e * Np;
    const double* ye = y + e * Np;
    const double* ze = z + e * Np;
    double* g = ggeo + e * 7 * Np;
    for (int k = 0; k < Nq; ++k)
      for (int j = 0; j < Nq; ++j)
        for (int i = 0; i < Nq; ++i) {
          double xr = 0, xs = 0, xt = 0, yr = 0, ys = 0, yt = 0, zr = 0, zs = 0, zt = 0;
          for (int m = 0; m < Nq; ++m) {
            int idr = m + Nq * (j + Nq * k);
            int ids = i + Nq * (m + Nq * k);
            int idt = i + Nq * (j + Nq * m);
            double dr = D[i * Nq + m], ds = D[j * Nq + m], dt = D[k * Nq + m];
            xr += dr * xe[idr]; xs += ds * xe[ids]; xt += dt * xe[idt];
            yr += dr * ye[idr]; ys += ds * ye[ids]; yt += dt * ye[idt];
            zr += dr * ze[idr]; zs += ds * ze[ids]; zt += dt * ze[idt];
          }
          double J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
          double rx = (ys * zt - zs * yt) / J, ry = -(xs * zt - zs * xt) / J, rz = (xs * yt - ys * xt) / J;
          double sx = -(yr * zt - zr * yt) / J, sy = (xr * zt - zr * xt) / J, sz = -(xr * yt - yr * xt) / J;
          double tx = (yr * zs - zr * ys) / J, ty = -(xr * zs - zr * xs) / J, tz = (xr * ys - yr * xs) / J;
          double JW = J * w1d[i] * w1d[j] * w1d[k];
          int n = i + Nq * (j + Nq * k);
          g[0 * Np + n] = JW;
          g[1 * Np + n] = JW * (rx * rx + ry * ry + rz * rz);
          g[2 * Np + n] = JW * (rx * sx + ry * sy + rz * sz);
          g[3 * Np + n] = JW * (rx * tx + ry * ty + rz * tz);
          g[4 * Np + n] = JW * (sx * sx + sy * sy + sz * sz);
          g[5 * Np + n] = JW * (sx * tx + sy * ty + sz * tz);
          g[6 * Np + n] = JW * (tx * tx + ty * ty + tz * tz);
        }
  }
}

/* ------------------------------------------------------------------------ */
/* axhelm: restates axhelm/kernel/CPU/axhelm.c (axhelm_v0 :27, axhelm_n3_v0   */
/* :113, axhelm_bk_v0 :229, axhelm_bk_n3_v0 :307) and the element list of the */
/* Partial OKL kernels (axhelm.okl:158,292,865,1188).  lambda0 = lambda[id],   */
/* lambda1 = lambda[id+offset]; the n3 variants share ggeo and lambda.        */
/* ------------------------------------------------------------------------ */
static void axhelm_element(int Nq, int64_t element, int64_t offset, int nf, int bk,
                           const double* ggeo, const double* D, const double* lambda,
                           const double* q, double* Aq, double* work)
{
  const int Np = Nq * Nq * Nq;
  double* s_q = work;            /* nf*Np */
  double* s_Gqr = s_q + 3 * Np;  /* nf*Np */
  double* s_Gqs = s_Gqr + 3 * Np;
  double* s_Gqt = s_Gqs + 3 * Np;
  const int64_t ebase = element * Np;
  const int64_t gbase = element * 7 * (int64_t)Np;

  for (int f = 0; f < nf; ++f)
    for (int n = 0; n < Np; ++n) s_q[f * Np + n] = q[ebase + n + f * offset];

  for (int k = 0; k < Nq; ++k)
    for (int j = 0; j < Nq; ++j)
      for (int i = 0; i < Nq; ++i) {
        const int n = i + Nq * (j + Nq * k);
        const double G00 = ggeo[gbase + 1 * Np + n];
        const double G01 = ggeo[gbase + 2 * Np + n];
        const double G02 = ggeo[gbase + 3 * Np + n];
        const double G11 = ggeo[gbase + 4 * Np + n];
        const double G12 = ggeo[gbase + 5 * Np + n];
        const double G22 = ggeo[gbase + 6 * Np + n];
        const double lam0 = bk ? 1.0 : lambda[ebase + n];
        for (int f = 0; f < nf; ++f) {
          const double* sq = s_q + f * Np;
          double qr = 0, qs = 0, qt = 0;
          for (int m = 0; m < Nq; ++m) {
            qr += D[i * Nq + m] * sq[m + Nq * (j + Nq * k)];
            qs += D[j * Nq + m] * sq[i + Nq * (m + Nq * k)];
            qt += D[k * Nq + m] * sq[i + Nq * (j + Nq * m)];
          }
          double gr = G00 * qr + G01 * qs + G02 * qt;
          double gs = G01 * qr + G11 * qs + G12 * qt;
          double gt = G02 * qr + G12 * qs + G22 * qt;
          if (!bk) { gr *= lam0; gs *= lam0; gt *= lam0; }
          s_Gqr[f * Np + n] = gr;
          s_Gqs[f * Np + n] = gs;
          s_Gqt[f * Np + n] = gt;
        }
      }

  for (int k = 0; k < Nq; ++k)
    for (int j = 0; j < Nq; ++j)
      for (int i = 0; i < Nq; ++i) {
        const int n = i + Nq * (j + Nq * k);
        const double GwJ = ggeo[gbase + 0 * Np + n];
        const double lam1 = bk ? 0.0 : lambda[ebase + n + offset];
        for (int f = 0; f < nf; ++f) {
          double ar = 0, as = 0, at = 0;
          const double* gr = s_Gqr + f * Np;
          const double* gs = s_Gqs + f * Np;
          const double* gt = s_Gqt + f * Np;
          for (int m = 0; m < Nq; ++m) {
            ar += D[m * Nq + i] * gr[m + Nq * (j + Nq * k)];
            as += D[m * Nq + j] * gs[i + Nq * (m + Nq * k)];
            at += D[m * Nq + k] * gt[i + Nq * (j + Nq * m)];
          }
          double out = ar + as + at;
          if (!bk) out += GwJ * lam1 * s_q[f * Np + n];
          Aq[ebase + n + f * offset] = out;
        }
      }
}

void nekbo_axhelm(int Nq, int64_t Nelements, int64_t offset, int flags, const int32_t* elementList,
                  const double* ggeo, const double* D, const double* lambda, const double* q,
                  double* Aq)
{
  const int Np = Nq * Nq * Nq;
  const int nf = (flags & NEKBO_AX_N3) ? 3 : 1;
  const int bk = (flags & NEKBO_AX_BK) ? 1 : 0;
  double* work = (double*)malloc(sizeof(double) * 12 * Np);
  for (int64_t e = 0; e < Nelements; ++e) {
    int64_t element = (flags & NEKBO_AX_PARTIAL) ? (int64_t)elementList[e] : e;
    axhelm_element(Nq, element, offset, nf, bk, ggeo, D, lambda, q, Aq, work);
  }
  free(work);
}

void nekbo_axhelm_omp(int Nq, int64_t Nelements, int64_t offset, int flags, const double* ggeo,
                      const double* D, const double* lambda, const double* q, double* Aq)
{
  const int Np = Nq * Nq * Nq;
  const int nf = (flags & NEKBO_AX_N3) ? 3 : 1;
  const int bk = (flags & NEKBO_AX_BK) ? 1 : 0;
#pragma omp parallel
  {
    double* work = (double*)malloc(sizeof(double) * 12 * Np);
#pragma omp for schedule(static)
    for (int64_t e = 0; e < Nelements; ++e)
      axhelm_element(Nq, e, offset, nf, bk, ggeo, D, lambda, q, Aq, work);
    free(work);
  }
}

int nekbo_omp_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* ogs: local branch of ogsSetup (3rdParty/ogs/src/ogsSetup.cpp:137-212) and  */
/* invDegree (:325-352).  Nodes with id 0 are skipped (:127,145).  Nodes are  */
/* sorted by (|id|, localId) (:40-52,156) and a new gather node starts at     */
/* every change of the signed id in that order (:161-166), so a run such as   */
/* 5, -5, 5 makes three gather nodes; gather nodes are then numbered in order */
/* of their first (lowest) local index (:173-189); each group lists its       */
/* members in ascending local index (:197-205).                               */
/* ------------------------------------------------------------------------ */
typedef struct {
  int64_t localId;
  int64_t baseId;
  int64_t newId;
  int owned;
} onode_t;

static int cmp_base(const void* a, const void* b)
{
  const onode_t* fa = (const onode_t*)a;
  const onode_t* fb = (const onode_t*)b;
  int64_t ia = fa->baseId < 0 ? -fa->baseId : fa->baseId;
  int64_t ib = fb->baseId < 0 ? -fb->baseId : fb->baseId;
  if (ia < ib) return -1;
  if (ia > ib) return +1;
  if (fa->localId < fb->localId) return -1;
  if (fa->localId > fb->localId) return +1;
  return 0;
}

static int cmp_local(const void* a, const void* b)
{
  const onode_t* fa = (const onode_t*)a;
  const onode_t* fb = (const onode_t*)b;
  if (fa->localId < fb->localId) return -1;
  if (fa->localId > fb->localId) return +1;
  return 0;
}

int64_t nekbo_ogs_setup(int64_t N, const int64_t* ids, int32_t* offsets, int32_t* gatherIds,
                        double* invDegree)
{
  int64_t Nlocal = 0;
  for (int64_t i = 0; i < N; ++i)
    if (ids[i] != 0) Nlocal++;
  for (int64_t n = 0; n < N; ++n) invDegree[n] = 1.0;
  offsets[0] = 0;
  if (Nlocal == 0) return 0;

  onode_t* nodes = (onode_t*)calloc((size_t)Nlocal, sizeof(onode_t));
  int64_t cnt = 0;
  for (int64_t i = 0; i < N; ++i) {
    if (ids[i] == 0) continue;
    nodes[cnt].localId = i;
    nodes[cnt].baseId = ids[i];
    nodes[cnt].owned = 0;
    cnt++;
  }
  qsort(nodes, (size_t)Nlocal, sizeof(onode_t), cmp_base);

  int64_t Ngather = 0;
  nodes[0].newId = 0;
  nodes[0].owned = 1;
  for (int64_t i = 1; i < Nlocal; ++i) {
    int s = 0;
    /* the sort keys on |id|, but a group ends wherever the SIGNED id changes
     * (ogsSetup.cpp:161-166): ids 5 and -5 never share a group */
    if (nodes[i].baseId != nodes[i - 1].baseId) { Ngather++; s = 1; }
    nodes[i].newId = Ngather;
    nodes[i].owned = s;
  }
  Ngather++;
  qsort(nodes, (size_t)Nlocal, sizeof(onode_t), cmp_local);

  int64_t* counts = (int64_t*)calloc((size_t)Ngather, sizeof(int64_t));
  int64_t* map = (int64_t*)calloc((size_t)Ngather, sizeof(int64_t));
  cnt = 0;
  for (int64_t i = 0; i < Nlocal; ++i) {
    int64_t newId = nodes[i].newId;
    if (nodes[i].owned) map[newId] = cnt++;
    nodes[i].newId = map[newId];
    counts[map[newId]]++;
  }
  free(map);
  for (int64_t g = 0; g < Ngather; ++g) {
    offsets[g + 1] = (int32_t)(offsets[g] + counts[g]);
    counts[g] = 0;
  }
  for (int64_t i = 0; i < Nlocal; ++i) {
    int64_t g = nodes[i].newId;
    gatherIds[offsets[g] + counts[g]] = (int32_t)nodes[i].localId;
    counts[g]++;
  }
  free(counts);
  free(nodes);

  /* invDegree = 1 / (scatter(gather(ones))) ; id-0 nodes keep 1 */
  for (int64_t g = 0; g < Ngather; ++g) {
    double deg = 0;
    for (int32_t n = offsets[g]; n < offsets[g + 1]; ++n) deg += 1.0;
    for (int32_t n = offsets[g]; n < offsets[g + 1]; ++n) invDegree[gatherIds[n]] = 1.0 / deg;
  }
  return Ngather;
}

/* gatherScatterMany_doubleAdd (3rdParty/ogs/okl/gatherScatterMany.okl:58-85):
 * for each group with more than one member, sum in CSR order and write the
 * sum back to every member; k fields at the given stride. */
void nekbo_gs_many_add(int64_t Ngather, const int32_t* offsets, const int32_t* gatherIds, int k,
                       int64_t stride, double* q)
{
  for (int f = 0; f < k; ++f)
    for (int64_t g = 0; g < Ngather; ++g) {
      const int32_t start = offsets[g], end = offsets[g + 1];
      if (start + 1 == end) continue;
      double gq = 0;
      for (int32_t n = start; n < end; ++n) gq += q[gatherIds[n] + f * stride];
      for (int32_t n = start; n < end; ++n) q[gatherIds[n] + f * stride] = gq;
    }
}

void nekbo_mask(int64_t Nmasked, const int32_t* maskIds, double* q)
{
  for (int64_t n = 0; n < Nmasked; ++n) q[maskIds[n]] = 0.0;
}

/* ------------------------------------------------------------------------ */
/* updateJacobi (nekBone/kernel/updateJacobi.okl:27-108): diagonal of the     */
/* element Helmholtz matrix; nodes with mapB==1 get 1.                         */
/* ------------------------------------------------------------------------ */
void nekbo_update_jacobi(int Nq, int64_t Nelements, int64_t offset, const int32_t* mapB,
                         const double* ggeo, const double* D, const double* lambda, double* diag)
{
  const int Np = Nq * Nq * Nq;
  for (int64_t e = 0; e < Nelements; ++e) {
    const int64_t gb = e * 7 * (int64_t)Np;
    for (int k = 0; k < Nq; ++k)
      for (int j = 0; j < Nq; ++j)
        for (int i = 0; i < Nq; ++i) {
          const int n = i + Nq * (j + Nq * k);
          const int64_t id = e * Np + n;
          double r_q = 1.0;
          if (!(mapB && mapB[id] == 1)) {
            const double grs = ggeo[gb + 2 * Np + n];
            const double grt = ggeo[gb + 3 * Np + n];
            const double gst = ggeo[gb + 5 * Np + n];
            const double gwJ = ggeo[gb + 0 * Np + n];
            const double l1 = lambda[id + offset];
            const double l0 = lambda[id];
            const double Dii = D[i * Nq + i], Djj = D[j * Nq + j], Dkk = D[k * Nq + k];
            r_q = 0.0;
            r_q += 2.0 * grs * l0 * Dii * Djj;
            r_q += 2.0 * grt * l0 * Dii * Dkk;
            r_q += 2.0 * gst * l0 * Djj * Dkk;
            for (int m = 0; m < Nq; ++m) {
              const int nr = m + Nq * (j + Nq * k);
              const int ns = i + Nq * (m + Nq * k);
              const int nt = i + Nq * (j + Nq * m);
              r_q += ggeo[gb + 1 * Np + nr] * lambda[e * Np + nr] * D[m * Nq + i] * D[m * Nq + i];
              r_q += ggeo[gb + 4 * Np + ns] * lambda[e * Np + ns] * D[m * Nq + j] * D[m * Nq + j];
              r_q += ggeo[gb + 6 * Np + nt] * lambda[e * Np + nt] * D[m * Nq + k] * D[m * Nq + k];
            }
            r_q += gwJ * l1;
          }
          diag[id] = r_q;
        }
  }
}

/* ------------------------------------------------------------------------ */
/* nekBone PCG                                                               */
/* ------------------------------------------------------------------------ */
double nekbo_wdot(int64_t N, int Nfields, int64_t offset, const double* w, const double* a,
                  const double* b)
{
  double s = 0;
  for (int f = 0; f < Nfields; ++f)
    for (int64_t i = 0; i < N; ++i) s += a[i + f * offset] * b[i + f * offset] * w[i];
  return s;
}

/* BPAxOperator (nekBone/solve.cpp:181-235) without overlap: axhelm, then the
 * gather-scatter (oogs start/finish), then the Dirichlet mask. */
void nekbo_bp_apply(const nekbo_bp* bp, const double* q, double* Aq)
{
  int flags = (bp->bk ? NEKBO_AX_BK : 0) | (bp->Nfields == 3 ? NEKBO_AX_N3 : 0);
  nekbo_axhelm(bp->Nq, bp->Nelements, bp->offset, flags, NULL, bp->ggeo, bp->D, bp->lambda, q, Aq);
  nekbo_gs_many_add(bp->Ngather, bp->gatherOffsets, bp->gatherIds, bp->Nfields, bp->offset, Aq);
  for (int f = 0; f < bp->Nfields; ++f) nekbo_mask(bp->Nmasked, bp->maskIds, Aq + f * bp->offset);
}

/* BPPCG (nekBone/solve.cpp:44-113) with BPPreconditioner (:167-179),
 * BPWeightedInnerProduct2 (:261-287), BPWeightedInnerProduct (:237-259),
 * BPScaledAdd (:289-293), BPUpdatePCG (:136-142) and updateJacobi (:146-165). */
void nekbo_zero_mean(int64_t Nloc, int Nfields, int64_t offset, double* q)
{
  double sum = 0.0;
  for (int64_t i = 0; i < Nloc; ++i)
    for (int f = 0; f < Nfields; ++f) sum += q[i + f * offset];
  const double mean = sum / (double)(Nloc * Nfields);
  for (int64_t i = 0; i < Nfields * offset; ++i) q[i] += -mean;
}

int nekbo_pcg(const nekbo_bp* bp, double* r, double* x, double tol, int maxit, int precond,
              int flexible, int fixed_iterations, double* rdotr_hist)
{
  const int64_t Nloc = bp->Nelements * (int64_t)bp->Nq * bp->Nq * bp->Nq;
  const int64_t Nall = bp->Nfields * bp->offset;
  double* p = (double*)calloc((size_t)Nall, sizeof(double));
  double* z = (double*)calloc((size_t)Nall, sizeof(double));
  double* Ap = (double*)calloc((size_t)Nall, sizeof(double));
  double* Ax = (double*)calloc((size_t)Nall, sizeof(double));
  double* invDiag = NULL;
  const double* w = bp->invDegree;

  double rdotz1 = 1, rdotz2 = 0, alpha = 0, beta = 0, TOL = 0;

  nekbo_bp_apply(bp, x, Ax);
  for (int64_t n = 0; n < Nall; ++n) r[n] = -1.0 * Ax[n] + 1.0 * r[n];

  if (precond == 1) {
    int32_t* mapB = (int32_t*)calloc((size_t)Nloc, sizeof(int32_t));
    for (int64_t m = 0; m < bp->Nmasked; ++m) mapB[bp->maskIds[m]] = 1;
    invDiag = (double*)calloc((size_t)Nall, sizeof(double));
    double* lam = NULL;
    const double* lamp = bp->lambda;
    if (bp->bk) { /* BK: lambda0 = 1, lambda1 = 0 */
      lam = (double*)calloc((size_t)(2 * bp->offset), sizeof(double));
      for (int64_t n = 0; n < bp->offset; ++n) lam[n] = 1.0;
      lamp = lam;
    }
    nekbo_update_jacobi(bp->Nq, bp->Nelements, bp->offset, mapB, bp->ggeo, bp->D, lamp, invDiag);
    nekbo_gs_many_add(bp->Ngather, bp->gatherOffsets, bp->gatherIds, 1, bp->offset, invDiag);
    for (int64_t n = 0; n < Nloc; ++n) invDiag[n] = 1.0 / invDiag[n];
    free(mapB);
    free(lam);
  }

  int iter;
  for (iter = 1; iter <= maxit; ++iter) {
    if (precond == 1) {
      /* the Jacobi diagonal of the shared operator serves every field */
      for (int f = 0; f < bp->Nfields; ++f)
        for (int64_t i = 0; i < Nloc; ++i) z[i + f * bp->offset] = invDiag[i] * r[i + f * bp->offset];
    } else {
      memcpy(z, r, sizeof(double) * (size_t)Nall);
    }
    rdotz2 = rdotz1;
    double rdotr = 0;
    rdotz1 = 0;
    for (int f = 0; f < bp->Nfields; ++f)
      for (int64_t i = 0; i < Nloc; ++i) {
        const int64_t ii = i + f * bp->offset;
        rdotz1 += r[ii] * z[ii] * w[i];
        rdotr += r[ii] * r[ii] * w[i];
      }
    if (rdotr_hist) rdotr_hist[iter - 1] = rdotr;
    if (iter == 1) TOL = fmax(tol * tol * rdotr, tol * tol);
    if (rdotr <= TOL && !fixed_iterations) break;

    if (flexible) {
      double zdotAp = nekbo_wdot(Nloc, bp->Nfields, bp->offset, w, z, Ap);
      beta = -alpha * zdotAp / rdotz2;
    } else {
      beta = (iter == 1) ? 0 : rdotz1 / rdotz2;
    }
    for (int64_t n = 0; n < Nall; ++n) p[n] = 1.0 * z[n] + beta * p[n];
    nekbo_bp_apply(bp, p, Ap);
    double pAp = nekbo_wdot(Nloc, bp->Nfields, bp->offset, w, p, Ap);
    alpha = rdotz1 / pAp;
    for (int64_t n = 0; n < Nall; ++n) {
      x[n] = x[n] + alpha * p[n];
      r[n] = r[n] - alpha * Ap[n];
    }
  }
  free(p); free(z); free(Ap); free(Ax); free(invDiag);
  return iter - 1;
}

/* The same BPPCG on all host threads: the reference's CPU path for this loop
 * (the OpenMP CPU axhelm of axhelm/kernel/CPU/axhelm.c, the gather-scatter and
 * the vector kernels of nekBone/kernel/utils.okl run by OCCA's OpenMP
 * backend).  Every loop over nodes, elements or gather groups is an OpenMP
 * loop (the groups are disjoint, so they run in parallel without races); the
 * inner products are OpenMP reductions, so their rounding differs from
 * nekbo_pcg's ordered sums.  A timing baseline for the CPU, never a parity
 * reference. */
static void gs_many_add_omp(int64_t Ngather, const int32_t* offsets, const int32_t* gatherIds, int k,
                            int64_t stride, double* q)
{
  for (int f = 0; f < k; ++f) {
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < Ngather; ++g) {
      const int32_t start = offsets[g], end = offsets[g + 1];
      if (start + 1 == end) continue;
      double gq = 0;
      for (int32_t n = start; n < end; ++n) gq += q[gatherIds[n] + f * stride];
      for (int32_t n = start; n < end; ++n) q[gatherIds[n] + f * stride] = gq;
    }
  }
}

/* The timed OpenMP PCG may take its single-field operator from the CPU
 * baseline build (cpu_axhelm.c: compile-time order, the reference's -O3);
 * only the benchmark installs it, the checker's paths never use it. */
static nekbo_cpu_axhelm_fn g_cpu_axhelm = 0;

void nekbo_set_cpu_axhelm(nekbo_cpu_axhelm_fn fn) { g_cpu_axhelm = fn; }

static void bp_apply_omp(const nekbo_bp* bp, const double* q, double* Aq)
{
  const int flags = (bp->bk ? NEKBO_AX_BK : 0) | (bp->Nfields == 3 ? NEKBO_AX_N3 : 0);
  if (!(g_cpu_axhelm && bp->Nfields == 1 &&
        g_cpu_axhelm(bp->Nq, bp->bk, bp->Nelements, bp->offset, bp->ggeo, bp->D, bp->lambda, q,
                     Aq) == 0))
    nekbo_axhelm_omp(bp->Nq, bp->Nelements, bp->offset, flags, bp->ggeo, bp->D, bp->lambda, q, Aq);
  gs_many_add_omp(bp->Ngather, bp->gatherOffsets, bp->gatherIds, bp->Nfields, bp->offset, Aq);
  for (int f = 0; f < bp->Nfields; ++f) {
    double* a = Aq + f * bp->offset;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < bp->Nmasked; ++n) a[bp->maskIds[n]] = 0.0;
  }
}

int nekbo_pcg_omp(const nekbo_bp* bp, double* r, double* x, double tol, int maxit, int precond,
                  int fixed_iterations, double* setup_s)
{
  const double t0 = omp_get_wtime();
  const int64_t Nloc = bp->Nelements * (int64_t)bp->Nq * bp->Nq * bp->Nq;
  const int64_t Nall = bp->Nfields * bp->offset;
  const int NF = bp->Nfields;
  const int64_t off = bp->offset;
  double* p = (double*)calloc((size_t)Nall, sizeof(double));
  double* z = (double*)calloc((size_t)Nall, sizeof(double));
  double* Ap = (double*)calloc((size_t)Nall, sizeof(double));
  double* Ax = (double*)calloc((size_t)Nall, sizeof(double));
  double* invDiag = NULL;
  const double* w = bp->invDegree;
  double rdotz1 = 1, rdotz2 = 0, alpha = 0, beta = 0, TOL = 0;

  bp_apply_omp(bp, x, Ax);
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < Nall; ++n) r[n] = r[n] - Ax[n];
  if (precond == 1) {
    int32_t* mapB = (int32_t*)calloc((size_t)Nloc, sizeof(int32_t));
    for (int64_t m = 0; m < bp->Nmasked; ++m) mapB[bp->maskIds[m]] = 1;
    invDiag = (double*)calloc((size_t)Nloc, sizeof(double));
    double* lam = NULL;
    const double* lamp = bp->lambda;
    if (bp->bk) {
      lam = (double*)calloc((size_t)(2 * off), sizeof(double));
      for (int64_t n = 0; n < off; ++n) lam[n] = 1.0;
      lamp = lam;
    }
    nekbo_update_jacobi(bp->Nq, bp->Nelements, off, mapB, bp->ggeo, bp->D, lamp, invDiag);
    gs_many_add_omp(bp->Ngather, bp->gatherOffsets, bp->gatherIds, 1, off, invDiag);
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < Nloc; ++n) invDiag[n] = 1.0 / invDiag[n];
    free(mapB);
    free(lam);
  }
  if (setup_s) *setup_s = omp_get_wtime() - t0;

  int iter;
  for (iter = 1; iter <= maxit; ++iter) {
    double rdotr = 0, rz = 0;
    for (int f = 0; f < NF; ++f) {
      double* zf = z + f * off;
      const double* rf = r + f * off;
#pragma omp parallel for schedule(static) reduction(+ : rz, rdotr)
      for (int64_t i = 0; i < Nloc; ++i) {
        const double zi = precond == 1 ? invDiag[i] * rf[i] : rf[i];
        zf[i] = zi;
        rz += rf[i] * zi * w[i];
        rdotr += rf[i] * rf[i] * w[i];
      }
    }
    rdotz2 = rdotz1;
    rdotz1 = rz;
    if (iter == 1) TOL = fmax(tol * tol * rdotr, tol * tol);
    if (rdotr <= TOL && !fixed_iterations) break;
    beta = (iter == 1) ? 0 : rdotz1 / rdotz2;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < Nall; ++n) p[n] = z[n] + beta * p[n];
    bp_apply_omp(bp, p, Ap);
    double pAp = 0;
    for (int f = 0; f < NF; ++f) {
      const double* pf = p + f * off;
      const double* af = Ap + f * off;
#pragma omp parallel for schedule(static) reduction(+ : pAp)
      for (int64_t i = 0; i < Nloc; ++i) pAp += pf[i] * af[i] * w[i];
    }
    alpha = rdotz1 / pAp;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < Nall; ++n) {
      x[n] = x[n] + alpha * p[n];
      r[n] = r[n] - alpha * Ap[n];
    }
  }
  free(p); free(z); free(Ap); free(Ax); free(invDiag);
  return iter - 1;
}

/* ------------------------------------------------------------------------ */
/* learned element preconditioner: 3x3x3 convolutions on the Nq^3 nodes of   */
/* each element with zero padding, tanh-form GELU.                            */
/* ------------------------------------------------------------------------ */
void nekbo_conv3d_forward(int Nq, int64_t Nelem, int Cin, int Cout, const float* W, const float* in,
                          float* out)
{
  const int Np = Nq * Nq * Nq;
  for (int64_t e = 0; e < Nelem; ++e)
    for (int co = 0; co < Cout; ++co)
      for (int k = 0; k < Nq; ++k)
        for (int j = 0; j < Nq; ++j)
          for (int i = 0; i < Nq; ++i) {
            double acc = 0.0;
            for (int ci = 0; ci < Cin; ++ci) {
              const float* src = in + (e * Cin + ci) * Np;
              const float* wk = W + ((int64_t)co * Cin + ci) * 27;
              for (int dk = -1; dk <= 1; ++dk)
                for (int dj = -1; dj <= 1; ++dj)
                  for (int di = -1; di <= 1; ++di) {
                    int ii = i + di, jj = j + dj, kk = k + dk;
                    if (ii < 0 || jj < 0 || kk < 0 || ii >= Nq || jj >= Nq || kk >= Nq) continue;
                    acc += (double)wk[(di + 1) + 3 * ((dj + 1) + 3 * (dk + 1))] *
                           (double)src[ii + Nq * (jj + Nq * kk)];
                  }
            }
            out[(e * Cout + co) * Np + i + Nq * (j + Nq * k)] = (float)acc;
          }
}

void nekbo_conv3d_backward(int Nq, int64_t Nelem, int Cin, int Cout, const float* W, const float* in,
                           const float* gout, float* gin, float* gW)
{
  const int Np = Nq * Nq * Nq;
  double* gWacc = (double*)calloc((size_t)Cout * Cin * 27, sizeof(double));
  for (int64_t e = 0; e < Nelem; ++e) {
    if (gin)
      for (int ci = 0; ci < Cin; ++ci)
        for (int n = 0; n < Np; ++n) gin[(e * Cin + ci) * Np + n] = 0.0f;
    for (int ci = 0; ci < Cin; ++ci)
      for (int k = 0; k < Nq; ++k)
        for (int j = 0; j < Nq; ++j)
          for (int i = 0; i < Nq; ++i) {
            double acc = 0.0;
            const float xin = in[(e * Cin + ci) * Np + i + Nq * (j + Nq * k)];
            for (int co = 0; co < Cout; ++co) {
              const float* go = gout + (e * Cout + co) * Np;
              const float* wk = W + ((int64_t)co * Cin + ci) * 27;
              double* gwk = gWacc + ((int64_t)co * Cin + ci) * 27;
              /* output node o = input node - tap offset */
              for (int dk = -1; dk <= 1; ++dk)
                for (int dj = -1; dj <= 1; ++dj)
                  for (int di = -1; di <= 1; ++di) {
                    int oi = i - di, oj = j - dj, ok = k - dk;
                    if (oi < 0 || oj < 0 || ok < 0 || oi >= Nq || oj >= Nq || ok >= Nq) continue;
                    const int tap = (di + 1) + 3 * ((dj + 1) + 3 * (dk + 1));
                    const double g = go[oi + Nq * (oj + Nq * ok)];
                    acc += (double)wk[tap] * g;
                    gwk[tap] += g * (double)xin;
                  }
            }
            if (gin) gin[(e * Cin + ci) * Np + i + Nq * (j + Nq * k)] = (float)acc;
          }
  }
  for (int64_t t = 0; t < (int64_t)Cout * Cin * 27; ++t) gW[t] += (float)gWacc[t];
  free(gWacc);
}

static double gelu_d(double x)
{
  const double c = 0.7978845608028654; /* sqrt(2/pi) */
  return 0.5 * x * (1.0 + tanh(c * (x + 0.044715 * x * x * x)));
}

void nekbo_gelu_forward(int64_t n, const float* x, float* y)
{
  for (int64_t i = 0; i < n; ++i) y[i] = (float)gelu_d(x[i]);
}

void nekbo_gelu_backward(int64_t n, const float* x, const float* gy, float* gx)
{
  const double c = 0.7978845608028654;
  for (int64_t i = 0; i < n; ++i) {
    const double v = x[i];
    const double u = c * (v + 0.044715 * v * v * v);
    const double t = tanh(u);
    const double du = c * (1.0 + 3.0 * 0.044715 * v * v);
    const double d = 0.5 * (1.0 + t) + 0.5 * v * (1.0 - t * t) * du;
    gx[i] = (float)(gy[i] * d);
  }
}

/* ---- dot benchmark: dot/kernel/VOLTA/dot.okl:27-169 ----
 * Each block fills s[t] (the weighted triple product of node b*B + t, 0 past
 * N; dot.okl:36-39, 77-85, 128-137), then halves it in place: s[t] += s[t+h]
 * for t < h.  Every step writes only below h and reads only at h or above, so
 * running the threads of a step one after the other is the same as running
 * them together. */
int64_t nekbo_dot_partials(int variant, int64_t N, int Nfields, int64_t offset, int blockSize,
                           const double* w, const double* x, const double* y, double* wxy)
{
  if (variant < 0 || variant > 2 || N < 0) return -1;
  if (blockSize != 256 && blockSize != 512 && blockSize != 1024) return -1;
  if (variant == 1 && blockSize != 256) return -1;
  const int NF = variant == 2 ? Nfields : 1;
  if (NF < 1 || NF > 3 || (NF > 1 && offset < N)) return -1;
  const int B = blockSize;
  const int64_t nblock = (N + B - 1) / B;
  double s[1024];
  for (int64_t b = 0; b < nblock; ++b) {
    for (int t = 0; t < B; ++t) {
      const int64_t id = t + (int64_t)B * b;
      if (variant == 2) { /* dot.okl:79-84 */
        double res = 0.0;
        if (id < N)
          for (int f = 0; f < NF; ++f) res += w[id + f * offset] * x[id + f * offset] * y[id + f * offset];
        s[t] = res;
      } else {
        s[t] = id < N ? w[id] * x[id] * y[id] : 0.0;
      }
    }
    if (variant == 1) { /* dot.okl:141-167: 8 groups of 32, then the group sums */
      double sb[8];
      for (int g = 0; g < 8; ++g) {
        double* a = s + 32 * g;
        for (int h = 16; h >= 2; h >>= 1)
          for (int t = 0; t < h; ++t) a[t] += a[t + h];
        sb[g] = a[0] + a[1];
      }
      for (int h = 4; h >= 1; h >>= 1)
        for (int t = 0; t < h; ++t) sb[t] += sb[t + h];
      wxy[b] = sb[0];
    } else { /* dot.okl:41-63 */
      for (int h = B / 2; h >= 2; h >>= 1)
        for (int t = 0; t < h; ++t) s[t] += s[t + h];
      wxy[b] = s[0] + s[1];
    }
  }
  return nblock;
}

/* ---- adv benchmark: advCubatureHex3D_v0, adv/kernel/VOLTA/adv.okl:27-261 ----
 * Same loop structure as the kernel: for each GLL plane c the r and s
 * interpolations (adv.okl:86-115) and the progressive t accumulation
 * (:117-123); derivatives and the advection term per cubature node
 * (:133-197); then per GLL plane c the t, s and r projections and the inverse
 * mass (:199-259). */
void nekbo_adv_cubature(int Nq, int cubNq, int64_t Nelements, const double* vgeo,
                        const double* cubvgeo, const double* cubD, const double* cubInterpT,
                        int64_t offset, const double* U, double* NU)
{
  enum { RX = 0, RY = 1, SX = 2, SY = 3, JW = 5, IJW = 6, RZ = 7, SZ = 8, TX = 9, TY = 10, TZ = 11, NV = 12 };
  const int Np = Nq * Nq * Nq, cq = cubNq, cNp = cq * cq * cq;
  double* Uc = (double*)malloc(sizeof(double) * 3 * cNp);
  double* A = (double*)malloc(sizeof(double) * 3 * cNp);
  double* T1 = (double*)malloc(sizeof(double) * 3 * Nq * cq);
  double* P1 = (double*)malloc(sizeof(double) * 3 * cq * cq);
#define I_(a, i) cubInterpT[(a) * cq + (i)]
#define D_(i, n) cubD[(i) * cq + (n)]
  for (int64_t e = 0; e < Nelements; ++e) {
    for (int n = 0; n < 3 * cNp; ++n) Uc[n] = 0.0;
    for (int c = 0; c < Nq; ++c) {
      for (int f = 0; f < 3; ++f)
        for (int b = 0; b < Nq; ++b)
          for (int i = 0; i < cq; ++i) {
            double acc = 0.0;
            for (int a = 0; a < Nq; ++a) acc += I_(a, i) * U[f * offset + e * Np + c * Nq * Nq + b * Nq + a];
            T1[(f * Nq + b) * cq + i] = acc;
          }
      for (int f = 0; f < 3; ++f)
        for (int j = 0; j < cq; ++j)
          for (int i = 0; i < cq; ++i) {
            double u2 = 0.0;
            for (int b = 0; b < Nq; ++b) u2 += I_(b, j) * T1[(f * Nq + b) * cq + i];
            for (int k = 0; k < cq; ++k) Uc[f * cNp + (k * cq + j) * cq + i] += I_(c, k) * u2;
          }
    }
    for (int k = 0; k < cq; ++k)
      for (int j = 0; j < cq; ++j)
        for (int i = 0; i < cq; ++i) {
          double dr[3], ds[3], dt[3];
          for (int f = 0; f < 3; ++f) {
            const double* u = Uc + f * cNp;
            double ar = 0.0, as = 0.0, at = 0.0;
            for (int n = 0; n < cq; ++n) ar += D_(i, n) * u[(k * cq + j) * cq + n];
            for (int n = 0; n < cq; ++n) as += D_(j, n) * u[(k * cq + n) * cq + i];
            for (int n = 0; n < cq; ++n) at += D_(k, n) * u[(n * cq + j) * cq + i];
            dr[f] = ar;
            ds[f] = as;
            dt[f] = at;
          }
          const int64_t g = e * (int64_t)cNp * NV + (k * cq + j) * cq + i;
          const int node = (k * cq + j) * cq + i;
          const double un = Uc[node], vn = Uc[cNp + node], wn = Uc[2 * cNp + node];
          const double jw = cubvgeo[g + JW * cNp];
          const double Uhat = jw * (un * cubvgeo[g + RX * cNp] + vn * cubvgeo[g + RY * cNp] + wn * cubvgeo[g + RZ * cNp]);
          const double Vhat = jw * (un * cubvgeo[g + SX * cNp] + vn * cubvgeo[g + SY * cNp] + wn * cubvgeo[g + SZ * cNp]);
          const double What = jw * (un * cubvgeo[g + TX * cNp] + vn * cubvgeo[g + TY * cNp] + wn * cubvgeo[g + TZ * cNp]);
          for (int f = 0; f < 3; ++f) A[f * cNp + node] = Uhat * dr[f] + Vhat * ds[f] + What * dt[f];
        }
    for (int c = 0; c < Nq; ++c) {
      for (int f = 0; f < 3; ++f)
        for (int j = 0; j < cq; ++j)
          for (int i = 0; i < cq; ++i) {
            double acc = 0.0;
            for (int k = 0; k < cq; ++k) acc += I_(c, k) * A[f * cNp + (k * cq + j) * cq + i];
            P1[(f * cq + j) * cq + i] = acc;
          }
      for (int f = 0; f < 3; ++f)
        for (int b = 0; b < Nq; ++b)
          for (int i = 0; i < cq; ++i) {
            double acc = 0.0;
            for (int j = 0; j < cq; ++j) acc += I_(b, j) * P1[(f * cq + j) * cq + i];
            T1[(f * Nq + b) * cq + i] = acc;
          }
      for (int f = 0; f < 3; ++f)
        for (int b = 0; b < Nq; ++b)
          for (int a = 0; a < Nq; ++a) {
            double acc = 0.0;
            for (int i = 0; i < cq; ++i) acc += I_(a, i) * T1[(f * Nq + b) * cq + i];
            const int m = c * Nq * Nq + b * Nq + a;
            NU[f * offset + e * Np + m] = vgeo[e * (int64_t)Np * NV + IJW * Np + m] * acc;
          }
    }
  }
#undef I_
#undef D_
  free(Uc);
  free(A);
  free(T1);
  free(P1);
}
