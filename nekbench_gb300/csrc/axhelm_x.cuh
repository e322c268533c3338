// FP64-accurate axhelm computed on the FP32 pipes (double-float arithmetic).
//
// GB300 issues FP32 FMAs at 64x the FP64 rate, so an FP64 operator evaluated
// with native DFMA is bound by the FP64 pipe long before HBM.  This variant
// reads and writes FP64 arrays in the reference layout but represents every
// value as an unevaluated sum hi + lo of two floats (about 48 significant
// bits) and uses the error-free transformations of Dekker and Knuth:
//   TwoProd(a,b) = (a*b, fma(a,b,-a*b)),  TwoSum(a,b) = (s, (a-(s-bb))+(b-bb)),
// with contractions accumulated as in Ogita, Rump and Oishi's Dot2.
// FP64 inputs are split into (hi, lo) with integer operations on the IEEE-754
// bit pattern, and each output is rebuilt by one FP64 addition, so the FP64
// pipe carries one instruction per node instead of ~59.  The result agrees
// with the FP64 operator to a few units of 1e-14 (relative, max-norm); values
// must lie in the float exponent range (about 1e-30 .. 1e30).
#pragma once

#include "internal.h"

#include <climits>

namespace nekb {
namespace axx {

struct df {
  float hi, lo;
};

// double -> (hi, lo): hi = the double's sign, exponent and first 24 significant
// bits (truncated); lo = the remaining 29 bits rounded to 24, so hi + lo holds
// 48 bits of the double.  Range: |d| < 3.4e38 (float range).  Below 5e-23 the
// low part is dropped (absolute error < 3e-30) and below 1.2e-38 the value
// maps to 0.
__device__ __forceinline__ df split(double d)
{
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  const int e = (int)((hw >> 20) & 0x7ff);  // biased FP64 exponent
  const unsigned sign = hw & 0x80000000u;
  df r;
  r.hi = 0.f;
  r.lo = 0.f;
  if (e < 897) return r;                              // below the float range: 0
  if (e > 1150) {                                     // above the float range: inf
    r.hi = __uint_as_float(sign | 0x7f800000u);
    return r;
  }
  // 23 stored bits of hi: 20 from the high word, 3 from the low word
  const unsigned m23 = ((hw & 0xfffffu) << 3) | (lw >> 29);
  r.hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | m23);
  if (e >= 949) {
    // remaining 29 bits with weight 2^(e-1075); 2^(e-1075) is a normal float
    // (biased exponent e - 948 >= 1)
    const float frem = __uint2float_rn(lw & 0x1fffffffu);
    const float lo = frem * __uint_as_float((unsigned)(e - 948) << 23);
    r.lo = sign ? -lo : lo;
  }
  return r;
}

// float -> double without the conversion unit: rebias and shift
__device__ __forceinline__ double widen(float f)
{
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xff;
  if (e == 0) return 0.0;
  const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
  const unsigned long long bits =
      sign | ((unsigned long long)(e + 896) << 52) | ((unsigned long long)(b & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ double join(df x) { return widen(x.hi) + widen(x.lo); }

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ df fast_norm(float s, float c)
{
  df r;
  r.hi = s + c;
  r.lo = c - (r.hi - s);
  return r;
}

// compensated accumulator: value = S + c
struct acc2 {
  float S = 0.f, c = 0.f;
  // += a*b with a, b double-floats (the lo*lo term is below the precision)
  __device__ __forceinline__ void fma2(df a, df b)
  {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    float t;
    two_sum(S, p, S, t);
    c += t + e;
  }
  __device__ __forceinline__ void add(df a)
  {
    float t;
    two_sum(S, a.hi, S, t);
    c += t + a.lo;
  }
  __device__ __forceinline__ df get() const { return fast_norm(S, c); }
};

template <int NQ, int NF>
struct CfgX {
  static constexpr int NQ2 = NQ * NQ;
  static constexpr int NP = NQ2 * NQ;
  // per element: q, Gqr, Gqs as double-floats
  static constexpr int PER_EL = 3 * NF * NP * 8;
  static constexpr int CAP = 112 * 1024;
  static constexpr int nel_fit(int n) { return (n <= 1 || n * PER_EL <= CAP) ? n : nel_fit(n - 1); }
  static constexpr int NEL0 = (256 / NQ2) > 0 ? (256 / NQ2) : 1;
  static constexpr int NEL = nel_fit(NEL0);
  static constexpr int THREADS = ((NEL * NQ2 + 31) / 32) * 32;
  static constexpr int DPAD = NQ * (NQ + 1);
  static constexpr int SMEM = (DPAD + NEL * 3 * NF * NP) * 8;
};

template <int NQ, int NF, bool BK>
__global__ void __launch_bounds__(CfgX<NQ, NF>::THREADS)
k_axhelm_x(const AxArgs a)
{
  using C = CfgX<NQ, NF>;
  constexpr int NQ2 = C::NQ2, NP = C::NP, NEL = C::NEL, DS = NQ + 1;
  if (a.skip != nullptr && *a.skip != 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  df* s_D = reinterpret_cast<df*>(smem_raw);
  df* s_all = s_D + C::DPAD;

  const int tid = threadIdx.x;
  const int el = tid / NQ2;
  const int ij = tid - el * NQ2;
  const int i = ij % NQ;
  const int j = ij / NQ;
  const int64_t eidx = (int64_t)blockIdx.x * NEL + el;
  const bool active = (el < NEL) && (eidx < a.Nelements);
  const int64_t element = eidx;

  const double* Dg = static_cast<const double*>(a.D);
  for (int t = tid; t < NQ2; t += blockDim.x) {
    // D entries are O(N^2): split them exactly with FP64 arithmetic (once per CTA)
    const double d = Dg[t];
    df v;
    v.hi = __double2float_rn(d);
    v.lo = __double2float_rn(d - (double)v.hi);
    s_D[(t / NQ) * DS + (t % NQ)] = v;
  }
  const int elc = active ? el : 0;
  df* s_q = s_all + elc * 3 * NF * NP;
  df* s_Gr = s_q + NF * NP;
  df* s_Gs = s_Gr + NF * NP;

  // geometry of layer k+1 is requested while layer k is computed; layer 0
  // before the first barrier (the kernel is otherwise waiting on these loads)
  const double* ge = static_cast<const double*>(a.ggeo) + element * 7 * NP + ij;
  const double* lam = static_cast<const double*>(a.lambda);
  double gnext[7];
  if (active) {
#pragma unroll
    for (int sl = 0; sl < 6; ++sl) gnext[sl] = ge[(sl + 1) * NP];
    if (!BK) gnext[6] = lam[element * NP + ij];
  }

  df r_q[NF][NQ];
  if (active) {
    const double* qe = static_cast<const double*>(a.q) + element * NP + ij;
#pragma unroll
    for (int f = 0; f < NF; ++f)
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const df v = split(qe[f * a.offset + k * NQ2]);
        r_q[f][k] = v;
        s_q[f * NP + k * NQ2 + ij] = v;
      }
  }
  __syncthreads();

  df r_Gt[NF][NQ];
  if (active) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const int n = k * NQ2 + ij;
      double gcur[7];
#pragma unroll
      for (int sl = 0; sl < 7; ++sl) gcur[sl] = gnext[sl];
      if (k + 1 < NQ) {
#pragma unroll
        for (int sl = 0; sl < 6; ++sl) gnext[sl] = ge[(sl + 1) * NP + (k + 1) * NQ2];
        if (!BK) gnext[6] = lam[element * NP + n + NQ2];
      } else if (!BK) {  // phase 3 starts with layer 0's GwJ and lambda1
        gnext[0] = ge[0];
        gnext[1] = lam[element * NP + ij + a.offset];
      }
      const df G00 = split(gcur[0]);
      const df G01 = split(gcur[1]);
      const df G02 = split(gcur[2]);
      const df G11 = split(gcur[3]);
      const df G12 = split(gcur[4]);
      const df G22 = split(gcur[5]);
      df lam0;
      if (!BK) lam0 = split(gcur[6]);
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const df* sq = s_q + f * NP + k * NQ2;
        acc2 ar, as, at;
#pragma unroll
        for (int m = 0; m < NQ; ++m) {
          ar.fma2(s_D[i * DS + m], sq[j * NQ + m]);
          as.fma2(s_D[j * DS + m], sq[m * NQ + i]);
          at.fma2(s_D[k * DS + m], r_q[f][m]);
        }
        const df qr = ar.get(), qs = as.get(), qt = at.get();
        acc2 gr, gs, gt;
        gr.fma2(G00, qr); gr.fma2(G01, qs); gr.fma2(G02, qt);
        gs.fma2(G01, qr); gs.fma2(G11, qs); gs.fma2(G12, qt);
        gt.fma2(G02, qr); gt.fma2(G12, qs); gt.fma2(G22, qt);
        df vr = gr.get(), vs = gs.get(), vt = gt.get();
        if (!BK) {
          acc2 t1, t2, t3;
          t1.fma2(lam0, vr); t2.fma2(lam0, vs); t3.fma2(lam0, vt);
          vr = t1.get(); vs = t2.get(); vt = t3.get();
        }
        s_Gr[f * NP + n] = vr;
        s_Gs[f * NP + n] = vs;
        r_Gt[f][k] = vt;
      }
    }
  }
  __syncthreads();

  if (active) {
    double* Aqe = static_cast<double*>(a.Aq) + element * NP + ij;
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const int n = k * NQ2 + ij;
      df wl1;
      if (!BK) {
        const double gw = gnext[0], l1 = gnext[1];
        if (k + 1 < NQ) {
          gnext[0] = ge[(k + 1) * NQ2];
          gnext[1] = lam[element * NP + n + NQ2 + a.offset];
        }
        acc2 t;
        t.fma2(split(gw), split(l1));
        wl1 = t.get();
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const df* gr = s_Gr + f * NP + k * NQ2;
        const df* gs = s_Gs + f * NP + k * NQ2;
        acc2 out;
#pragma unroll
        for (int m = 0; m < NQ; ++m) {
          out.fma2(s_D[m * DS + i], gr[j * NQ + m]);
          out.fma2(s_D[m * DS + j], gs[m * NQ + i]);
          out.fma2(s_D[m * DS + k], r_Gt[f][m]);
        }
        if (!BK) out.fma2(wl1, r_q[f][k]);
        Aqe[f * a.offset + k * NQ2] = join(out.get());
      }
    }
  }
}

template <int NQ, int NF, bool BK>
int run(const AxArgs& a, cudaStream_t s)
{
  using C = CfgX<NQ, NF>;
  auto kern = k_axhelm_x<NQ, NF, BK>;
  static SmemOptIn smem_opt;
  NEKB_TRY(smem_opt.ensure(kern, C::SMEM));  // dynamic + static may pass 48 KB
  const int64_t nblk = (a.Nelements + C::NEL - 1) / C::NEL;
  if (nblk == 0) return NEKB_OK;
  if (nblk > INT_MAX) return fail(NEKB_ERR_INVALID, "axhelm: too many elements");
  kern<<<(unsigned)nblk, C::THREADS, C::SMEM, s>>>(a);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

template <int NQ>
int run_flags(int flags, const AxArgs& a, cudaStream_t s)
{
  if (flags & NEKB_AX_PARTIAL)
    return fail(NEKB_ERR_UNSUPPORTED, "axhelm: Partial variants run in NEKB_FP64");
  const bool bk = flags & NEKB_AX_BK, n3 = flags & NEKB_AX_N3;
  if (n3) return bk ? run<NQ, 3, true>(a, s) : run<NQ, 3, false>(a, s);
  return bk ? run<NQ, 1, true>(a, s) : run<NQ, 1, false>(a, s);
}

}  // namespace axx
}  // namespace nekb
