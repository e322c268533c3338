// The dealiased advection operator of nekBench's adv benchmark,
// advCubatureHex3D_v0 (adv/kernel/VOLTA/adv.okl:27-261), in FP64 (policy F64)
// or in double-float arithmetic on the FP32 pipes (policy DF):
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
// Where cubNq^2 <= 160 and two CTAs' shared memory fit on an SM, the FP64
// kernel's launch bounds ask for two CTAs per SM (the
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
#include "axhelm_x.cuh"
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
  // with the advection terms [f][k][j][i] staged in shared memory instead of registers
  static constexpr int bytes_adv = bytes + 8 * 3 * Cp;
  // two CTAs per SM: small CTAs whose shared memory fits twice in the SM's 228 KB
  static constexpr bool fits_twice(int b) { return threads <= 160 && 2 * (b + 1024) <= 228 * 1024; }
};

// Arithmetic of the kernel.  F64: native FP64 FMAs.  DF: every value an
// unevaluated sum hi + lo of two floats (about 48 significant bits), products
// and sums with error-free transformations on the FP32 pipes (axhelm_x.cuh);
// FP64 inputs are split with integer operations and each output rebuilt with
// one FP64 addition.  Values must lie in the float range (1e-30 .. 1e30).
struct F64 {
  using T = double;
  static constexpr __host__ __device__ bool adv_in_smem(int) { return false; }
  struct Acc {
    double v = 0.0;
    __device__ __forceinline__ void fma(double a, double b) { v = ::fma(a, b, v); }
    __device__ __forceinline__ double get() const { return v; }
  };
  static __device__ __forceinline__ double in(double d) { return d; }
  static __device__ __forceinline__ double in_exact(double d) { return d; }
  static __device__ __forceinline__ double out(double x) { return x; }
};

struct __align__(8) D2 {
  float hi, lo;
};

struct DF {
  using T = D2;
  // On cubature grids of 10^3 nodes and more, the advection terms go to shared
  // memory: the registers they free let two CTAs share an SM, which the
  // compensated sums' dependency chains need (N=7, cubN=11: 3.74 ms against
  // 8.13 ms with the terms in registers).  Smaller grids already run several
  // CTAs per SM and keep them in registers (N=7, cubN=7: 2.08 against 2.92 ms).
  static constexpr __host__ __device__ bool adv_in_smem(int cq) { return cq * cq > 96; }
  struct Acc {
    axx::acc2 a;
    __device__ __forceinline__ void fma(D2 x, D2 y) { a.fma2(axx::df{x.hi, x.lo}, axx::df{y.hi, y.lo}); }
    __device__ __forceinline__ D2 get() const
    {
      const axx::df r = a.get();
      return D2{r.hi, r.lo};
    }
  };
  static __device__ __forceinline__ D2 in(double d)
  {
    const axx::df r = axx::split(d);
    return D2{r.hi, r.lo};
  }
  // exact two-float split with FP64 arithmetic (operator matrices, once per CTA)
  static __device__ __forceinline__ D2 in_exact(double d)
  {
    const float hi = __double2float_rn(d);
    return D2{hi, __double2float_rn(d - (double)hi)};
  }
  static __device__ __forceinline__ double out(D2 x) { return axx::join(axx::df{x.hi, x.lo}); }
};

template <int NQ, int CQ, class P>
constexpr int adv_smem_bytes()
{
  return P::adv_in_smem(CQ) ? AdvShape<NQ, CQ>::bytes_adv : AdvShape<NQ, CQ>::bytes;
}

template <int NQ, int CQ, class P>
__global__ void __launch_bounds__(CQ * CQ, AdvShape<NQ, CQ>::fits_twice(adv_smem_bytes<NQ, CQ, P>()) ? 2 : 1)
k_adv_cubature(const double* __restrict__ vgeo, const double* __restrict__ cubvgeo,
               const double* __restrict__ cubD, const double* __restrict__ cubInterpT,
               int64_t offset, const double* __restrict__ U, double* __restrict__ NU)
{
  using S = AdvShape<NQ, CQ>;
  using T = typename P::T;
  using Acc = typename P::Acc;
  constexpr bool kAdvSmem = P::adv_in_smem(CQ);
  static_assert(sizeof(T) == 8, "shared-memory plan assumes 8-byte values");
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T* sI = reinterpret_cast<T*>(sm_raw);  // sI[a CQ + i] = I(i <- a)
  T* sD = sI + S::nI;                    // sD[i CQ + n]
  T* sU = sD + S::nD;                    // [f][c][b][a]
  T* sX = sU + S::nU;
  T* sY = sX + S::nX;
  T* sC = sX;                            // [f][k][j][i], over sX and sY
  T* sA = sX + S::nXY;                   // advection terms [f][k][j][i] (kAdvSmem)

  const int tid = threadIdx.x, i = tid % CQ, j = tid / CQ;
  const int64_t e = blockIdx.x;
  for (int n = tid; n < S::nI; n += S::threads) sI[n] = P::in_exact(cubInterpT[n]);
  for (int n = tid; n < S::nD; n += S::threads) sD[n] = P::in_exact(cubD[n]);
  for (int n = tid; n < S::nU; n += S::threads) {
    const int f = n / S::Np;
    sU[n] = P::in(U[f * offset + e * S::Np + (n - f * S::Np)]);
  }
  __syncthreads();

  // interpolate in r: X[f][c][b][i] = sum_a I(i <- a) U[f][c][b][a]
  for (int n = tid; n < S::nX; n += S::threads) {
    const int ii = n % CQ;
    const T* u = sU + (n / CQ) * NQ;
    Acc acc;
#pragma unroll
    for (int a = 0; a < NQ; ++a) acc.fma(sI[a * CQ + ii], u[a]);
    sX[n] = acc.get();
  }
  __syncthreads();
  // interpolate in s: Y[f][c][j][i] = sum_b I(j <- b) X[f][c][b][i]
  for (int n = tid; n < S::nY; n += S::threads) {
    const int ii = n % CQ, jj = (n / CQ) % CQ;
    const T* x = sX + (n / (CQ * CQ)) * NQ * CQ + ii;
    Acc acc;
#pragma unroll
    for (int b = 0; b < NQ; ++b) acc.fma(sI[b * CQ + jj], x[b * CQ]);
    sY[n] = acc.get();
  }
  __syncthreads();
  // interpolate in t along this thread's column: c[f][k] = sum_c I(k <- c) Y[f][c][j][i]
  T col[3][CQ];
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    T y[NQ];
#pragma unroll
    for (int c = 0; c < NQ; ++c) y[c] = sY[((f * NQ + c) * CQ + j) * CQ + i];
#pragma unroll
    for (int k = 0; k < CQ; ++k) {
      Acc acc;
#pragma unroll
      for (int c = 0; c < NQ; ++c) acc.fma(sI[c * CQ + k], y[c]);
      col[f][k] = acc.get();
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
  T adv[kAdvSmem ? 1 : 3][kAdvSmem ? 1 : CQ];
#pragma unroll
  for (int k = 0; k < CQ; ++k) {
    T dr[3], ds[3], dt[3], uc[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const T* c = sC + f * S::Cp;
      Acc ar, as, at;
#pragma unroll
      for (int n = 0; n < CQ; ++n) {
        ar.fma(sD[i * CQ + n], c[(k * CQ + j) * CQ + n]);
        as.fma(sD[j * CQ + n], c[(k * CQ + n) * CQ + i]);
        at.fma(sD[k * CQ + n], c[(n * CQ + j) * CQ + i]);
      }
      dr[f] = ar.get();
      ds[f] = as.get();
      dt[f] = at.get();
      uc[f] = c[(k * CQ + j) * CQ + i];
    }
    const double* gk = g + k * CQ * CQ;
    const T JW = P::in(gk[kJW * S::Cp]);
    constexpr int slot[3][3] = {{kRX, kRY, kRZ}, {kSX, kSY, kSZ}, {kTX, kTY, kTZ}};
    T hat[3];  // JW (u . grad r), JW (u . grad s), JW (u . grad t)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      Acc h;
#pragma unroll
      for (int f = 0; f < 3; ++f) h.fma(uc[f], P::in(gk[slot[d][f] * S::Cp]));
      Acc hj;
      hj.fma(JW, h.get());
      hat[d] = hj.get();
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      Acc a;
      a.fma(hat[0], dr[f]);
      a.fma(hat[1], ds[f]);
      a.fma(hat[2], dt[f]);
      if (kAdvSmem)
        sA[((f * CQ + k) * CQ + j) * CQ + i] = a.get();
      else
        adv[kAdvSmem ? 0 : f][kAdvSmem ? 0 : k] = a.get();
    }
  }
  __syncthreads();  // the cubature values are read: Y takes the t-projection

  // project in t: Y[f][c][j][i] = sum_k I(k <- c) adv[f][k]
#pragma unroll
  for (int f = 0; f < 3; ++f)
#pragma unroll
    for (int c = 0; c < NQ; ++c) {
      Acc acc;
#pragma unroll
      for (int k = 0; k < CQ; ++k)
        acc.fma(sI[c * CQ + k], kAdvSmem ? sA[((f * CQ + k) * CQ + j) * CQ + i]
                                              : adv[kAdvSmem ? 0 : f][kAdvSmem ? 0 : k]);
      sY[((f * NQ + c) * CQ + j) * CQ + i] = acc.get();
    }
  __syncthreads();
  // project in s: X[f][c][b][i] = sum_j I(j <- b) Y[f][c][j][i]
  for (int n = tid; n < S::nX; n += S::threads) {
    const int ii = n % CQ, b = (n / CQ) % NQ;
    const T* y = sY + (n / (CQ * NQ)) * CQ * CQ + ii;
    Acc acc;
#pragma unroll
    for (int jj = 0; jj < CQ; ++jj) acc.fma(sI[b * CQ + jj], y[jj * CQ]);
    sX[n] = acc.get();
  }
  __syncthreads();
  // project in r and apply the inverse mass: NU[f][c][b][a] = IJW sum_i I(i <- a) X[f][c][b][i]
  const double* ijw = vgeo + e * (int64_t)S::Np * kNvgeo + kIJW * S::Np;
  for (int n = tid; n < S::nU; n += S::threads) {
    const int f = n / S::Np, m = n - f * S::Np, a = m % NQ;
    const T* x = sX + (n / NQ) * CQ;
    Acc acc;
#pragma unroll
    for (int ii = 0; ii < CQ; ++ii) acc.fma(sI[a * CQ + ii], x[ii]);
    Acc scaled;
    scaled.fma(P::in(ijw[m]), acc.get());
    NU[f * offset + e * S::Np + m] = P::out(scaled.get());
  }
}

template <int NQ, int CQ, class P>
int launch_p(int64_t E, const double* vgeo, const double* cubvgeo, const double* cubD,
             const double* cubInterpT, int64_t offset, const double* U, double* NU, cudaStream_t s)
{
  using S = AdvShape<NQ, CQ>;
  constexpr int bytes = adv_smem_bytes<NQ, CQ, P>();
  static_assert(bytes <= 227 * 1024, "adv: shared memory plan exceeds 227 KB");
  static SmemOptIn smem_opt;
  NEKB_TRY(smem_opt.ensure(k_adv_cubature<NQ, CQ, P>, bytes));
  k_adv_cubature<NQ, CQ, P><<<(unsigned)E, S::threads, bytes, s>>>(vgeo, cubvgeo, cubD,
                                                                   cubInterpT, offset, U, NU);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

// split = false: native FP64; true: double-float on the FP32 pipes
template <int NQ, int CQ>
int launch(bool split, int64_t E, const double* vgeo, const double* cubvgeo, const double* cubD,
           const double* cubInterpT, int64_t offset, const double* U, double* NU, cudaStream_t s)
{
  return split ? launch_p<NQ, CQ, DF>(E, vgeo, cubvgeo, cubD, cubInterpT, offset, U, NU, s)
               : launch_p<NQ, CQ, F64>(E, vgeo, cubvgeo, cubD, cubInterpT, offset, U, NU, s);
}

}  // namespace adv
}  // namespace nekb
