// The dealiased advection operator of nekBench's adv benchmark,
// advCubatureHex3D_v0 (adv/kernel/VOLTA/adv.okl:27-261), in FP64:
//
//   NU_f = IJW . (I^T x I^T x I^T) [ Uhat dUc_f/dr + Vhat dUc_f/ds + What dUc_f/dt ]
//   Uc_f = (I x I x I) U_f,   Uhat = JW (Uc . grad r), Vhat = JW (Uc . grad s),
//   What = JW (Uc . grad t),  f = 0, 1, 2 (the three velocity components)
//
// with I(i <- a) = cubInterpT[a cubNq + i] (GLL node a to cubature node i),
// the cubature derivative d/dr = cubD[i cubNq + n] and the metric terms of
// cubvgeo / the inverse mass IJW of vgeo in the reference layout
// (slot s of element e at [e Nvgeo Np + s Np + node], core/params.h:2-13,63).
//
// The arithmetic is FP64 FMAs (about 0.36 M per element at N=7, cubN=11), and
// GB300 retires about two FP64 FMAs per clock per SM, so the kernel is bound
// by the FP64 pipe, not by HBM (about 166 KB per element, almost all of it the
// cubature metric terms).  The design therefore spends no extra FP64
// operation: one CTA of cubNq^2 threads per element; the element's three
// fields, the sum-factorised intermediates and the cubature values live in
// shared memory; every contraction is one FMA chain per output in the
// reference's summation order (r, then s, then t on the way in; t, s, r on
// the way out).  Thread (i, j) owns the cubature column (i, j, 0..cubNq-1) for
// the t-direction passes and the pointwise advection.
// Where cubNq^2 <= 160 the launch bounds ask for two CTAs per SM (the
// registers drop from 220 to 168 at cubNq = 12, with a 176-byte spill): the
// second CTA fills the FP64 pipe while the first waits at a barrier, 11 %
// faster at N=7, cubN=11 than one CTA per SM.
//
// The reference kernel stages the t-projected slice in s_U, declared
// Nq x Nq, but writes and reads it for all cubNq x cubNq (i, j)
// (adv.okl:203-231); for cubN > N those accesses run past the array.  Here the
// slice is cubNq x cubNq, i.e. the operator the reference's comment names
// (adv.okl:192).  For cubN = N the two agree.
#pragma once
#include "internal.h"

namespace nekb {
namespace adv {

// vgeo slots (core/params.h:2-13) and their count (core/params.h:63)
constexpr int kRX = 0, kRY = 1, kSX = 2, kSY = 3, kJW = 5, kIJW = 6, kRZ = 7, kSZ = 8, kTX = 9,
              kTY = 10, kTZ = 11, kNvgeo = 12;

template <int NQ, int CQ>
struct AdvShape {
  static constexpr int Np = NQ * NQ * NQ, Cp = CQ * CQ * CQ, threads = CQ * CQ;
  static constexpr int nI = NQ * CQ, nD = CQ * CQ, nU = 3 * Np;
  static constexpr int nX = 3 * NQ * NQ * CQ;  // [f][c][b][i]: r-interpolated, then s-projected
  static constexpr int nY = 3 * NQ * CQ * CQ;  // [f][c][j][i]: s-interpolated, then t-projected
  static constexpr int nXY = nX + nY > 3 * Cp ? nX + nY : 3 * Cp;  // cubature values [f][k][j][i]
  static constexpr int bytes = 8 * (nI + nD + nU + nXY);
};

template <int NQ, int CQ>
__global__ void __launch_bounds__(CQ * CQ, (CQ * CQ <= 160 ? 2 : 1))
k_adv_cubature(const double* __restrict__ vgeo, const double* __restrict__ cubvgeo,
               const double* __restrict__ cubD, const double* __restrict__ cubInterpT,
               int64_t offset, const double* __restrict__ U, double* __restrict__ NU)
{
  using S = AdvShape<NQ, CQ>;
  extern __shared__ __align__(16) double sm[];
  double* sI = sm;           // sI[a CQ + i] = I(i <- a)
  double* sD = sI + S::nI;   // sD[i CQ + n]
  double* sU = sD + S::nD;   // [f][c][b][a]
  double* sX = sU + S::nU;
  double* sY = sX + S::nX;
  double* sC = sX;           // [f][k][j][i], over sX and sY

  const int tid = threadIdx.x, i = tid % CQ, j = tid / CQ;
  const int64_t e = blockIdx.x;
  for (int n = tid; n < S::nI; n += S::threads) sI[n] = cubInterpT[n];
  for (int n = tid; n < S::nD; n += S::threads) sD[n] = cubD[n];
  for (int n = tid; n < S::nU; n += S::threads) {
    const int f = n / S::Np;
    sU[n] = U[f * offset + e * S::Np + (n - f * S::Np)];
  }
  __syncthreads();

  // interpolate in r: X[f][c][b][i] = sum_a I(i <- a) U[f][c][b][a]
  for (int n = tid; n < S::nX; n += S::threads) {
    const int ii = n % CQ;
    const double* u = sU + (n / CQ) * NQ;
    double acc = 0.0;
#pragma unroll
    for (int a = 0; a < NQ; ++a) acc = fma(sI[a * CQ + ii], u[a], acc);
    sX[n] = acc;
  }
  __syncthreads();
  // interpolate in s: Y[f][c][j][i] = sum_b I(j <- b) X[f][c][b][i]
  for (int n = tid; n < S::nY; n += S::threads) {
    const int ii = n % CQ, jj = (n / CQ) % CQ;
    const double* x = sX + (n / (CQ * CQ)) * NQ * CQ + ii;
    double acc = 0.0;
#pragma unroll
    for (int b = 0; b < NQ; ++b) acc = fma(sI[b * CQ + jj], x[b * CQ], acc);
    sY[n] = acc;
  }
  __syncthreads();
  // interpolate in t along this thread's column: c[f][k] = sum_c I(k <- c) Y[f][c][j][i]
  double col[3][CQ];
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    double y[NQ];
#pragma unroll
    for (int c = 0; c < NQ; ++c) y[c] = sY[((f * NQ + c) * CQ + j) * CQ + i];
#pragma unroll
    for (int k = 0; k < CQ; ++k) {
      double acc = 0.0;
#pragma unroll
      for (int c = 0; c < NQ; ++c) acc = fma(sI[c * CQ + k], y[c], acc);
      col[f][k] = acc;
    }
  }
  __syncthreads();  // X and Y are read: the cubature values take their place
#pragma unroll
  for (int f = 0; f < 3; ++f)
#pragma unroll
    for (int k = 0; k < CQ; ++k) sC[((f * CQ + k) * CQ + j) * CQ + i] = col[f][k];
  __syncthreads();

  // derivatives and the advection term at cubature node (i, j, k)
  const double* g = cubvgeo + e * (int64_t)S::Cp * kNvgeo + j * CQ + i;
  double adv[3][CQ];
#pragma unroll
  for (int k = 0; k < CQ; ++k) {
    double dr[3], ds[3], dt[3], uc[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const double* c = sC + f * S::Cp;
      double ar = 0.0, as = 0.0, at = 0.0;
#pragma unroll
      for (int n = 0; n < CQ; ++n) {
        ar = fma(sD[i * CQ + n], c[(k * CQ + j) * CQ + n], ar);
        as = fma(sD[j * CQ + n], c[(k * CQ + n) * CQ + i], as);
        at = fma(sD[k * CQ + n], c[(n * CQ + j) * CQ + i], at);
      }
      dr[f] = ar;
      ds[f] = as;
      dt[f] = at;
      uc[f] = c[(k * CQ + j) * CQ + i];
    }
    const double* gk = g + k * CQ * CQ;
    const double JW = gk[kJW * S::Cp];
    const double Uhat = JW * (uc[0] * gk[kRX * S::Cp] + uc[1] * gk[kRY * S::Cp] + uc[2] * gk[kRZ * S::Cp]);
    const double Vhat = JW * (uc[0] * gk[kSX * S::Cp] + uc[1] * gk[kSY * S::Cp] + uc[2] * gk[kSZ * S::Cp]);
    const double What = JW * (uc[0] * gk[kTX * S::Cp] + uc[1] * gk[kTY * S::Cp] + uc[2] * gk[kTZ * S::Cp]);
#pragma unroll
    for (int f = 0; f < 3; ++f) adv[f][k] = Uhat * dr[f] + Vhat * ds[f] + What * dt[f];
  }
  __syncthreads();  // the cubature values are read: Y takes the t-projection

  // project in t: Y[f][c][j][i] = sum_k I(k <- c) adv[f][k]
#pragma unroll
  for (int f = 0; f < 3; ++f)
#pragma unroll
    for (int c = 0; c < NQ; ++c) {
      double acc = 0.0;
#pragma unroll
      for (int k = 0; k < CQ; ++k) acc = fma(sI[c * CQ + k], adv[f][k], acc);
      sY[((f * NQ + c) * CQ + j) * CQ + i] = acc;
    }
  __syncthreads();
  // project in s: X[f][c][b][i] = sum_j I(j <- b) Y[f][c][j][i]
  for (int n = tid; n < S::nX; n += S::threads) {
    const int ii = n % CQ, b = (n / CQ) % NQ;
    const double* y = sY + (n / (CQ * NQ)) * CQ * CQ + ii;
    double acc = 0.0;
#pragma unroll
    for (int jj = 0; jj < CQ; ++jj) acc = fma(sI[b * CQ + jj], y[jj * CQ], acc);
    sX[n] = acc;
  }
  __syncthreads();
  // project in r and apply the inverse mass: NU[f][c][b][a] = IJW sum_i I(i <- a) X[f][c][b][i]
  const double* ijw = vgeo + e * (int64_t)S::Np * kNvgeo + kIJW * S::Np;
  for (int n = tid; n < S::nU; n += S::threads) {
    const int f = n / S::Np, m = n - f * S::Np, a = m % NQ;
    const double* x = sX + (n / NQ) * CQ;
    double acc = 0.0;
#pragma unroll
    for (int ii = 0; ii < CQ; ++ii) acc = fma(sI[a * CQ + ii], x[ii], acc);
    NU[f * offset + e * S::Np + m] = ijw[m] * acc;
  }
}

template <int NQ, int CQ>
int launch(int64_t E, const double* vgeo, const double* cubvgeo, const double* cubD,
           const double* cubInterpT, int64_t offset, const double* U, double* NU, cudaStream_t s)
{
  using S = AdvShape<NQ, CQ>;
  static bool configured = false;
  if (!configured) {
    NEKB_CUDA(cudaFuncSetAttribute(k_adv_cubature<NQ, CQ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   S::bytes));
    configured = true;
  }
  k_adv_cubature<NQ, CQ><<<(unsigned)E, S::threads, S::bytes, s>>>(vgeo, cubvgeo, cubD, cubInterpT,
                                                                   offset, U, NU);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

}  // namespace adv
}  // namespace nekb
