// Matrix-free Helmholtz operator on hexahedra of order NQ-1 (axhelm).
//
// Math (axhelm/kernel/CPU/axhelm.c:27-111, axhelm/axhelmReference.cpp:19-89):
//   qr,qs,qt = sum_m D[.][m] q(..m..)                         (3 contractions)
//   [Gqr,Gqs,Gqt] = lambda0 * G [qr,qs,qt]                  (G symmetric, 6 slots)
//   Aq = sum_m D[m][i] Gqr(m,j,k) + D[m][j] Gqs(i,m,k) + D[m][k] Gqt(i,j,m)
//        + GwJ * lambda1 * q                                  (omitted in BK mode)
//
// GPU mapping: one CTA holds NEL elements; thread (i,j) of an element owns the
// k-column of nodes (i,j,0..NQ-1).  The column of q and of Gqt stays in
// registers, so the t-direction contractions need no shared memory; the
// r- and s-direction contractions read the element's q (and Gqr/Gqs) slices
// from shared memory.  ggeo, lambda, q and Aq are read/written exactly once,
// coalesced along the (i,j) plane.  Two barriers per element.
//
// Precision modes: FP64; FP32; BF16 storage of ggeo/lambda with FP32
// arithmetic; FP32 with the geometry rebuilt on the fly from 24 trilinear
// coefficients per element (no ggeo traffic).
#pragma once

#include "internal.h"

#include <climits>

namespace nekb {
namespace ax {

template <int PREC> struct Prec;
template <> struct Prec<NEKB_FP64> { using T = double; using TG = double; };
template <> struct Prec<NEKB_FP32> { using T = float; using TG = float; };
template <> struct Prec<NEKB_BF16> { using T = float; using TG = __nv_bfloat16; };
template <> struct Prec<NEKB_FP32_TRILINEAR> { using T = float; using TG = float; };

__device__ __forceinline__ float to_c(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float to_c(float v) { return v; }
__device__ __forceinline__ double to_c(double v) { return v; }

template <int NQ, int NF, int PREC>
struct Cfg {
  using T = typename Prec<PREC>::T;
  static constexpr int NQ2 = NQ * NQ;
  static constexpr int NP = NQ2 * NQ;
  static constexpr int PER_EL = 3 * NF * NP * (int)sizeof(T);
  static constexpr int CAP = 112 * 1024;
  static constexpr int nel_fit(int n) { return (n <= 1 || n * PER_EL <= CAP) ? n : nel_fit(n - 1); }
  static constexpr int NEL0 = (256 / NQ2) > 0 ? (256 / NQ2) : 1;
  static constexpr int NEL = nel_fit(NEL0);
  static constexpr int THREADS = ((NEL * NQ2 + 31) / 32) * 32;
  static constexpr int DPAD = ((NQ * (NQ + 1) + 3) / 4) * 4;  // D, rows padded to NQ+1
  static constexpr bool TRI = (PREC == NEKB_FP32_TRILINEAR);
  // two CTAs per SM for the 4-byte single-field kernels (caps registers at 128)
  static constexpr int MINB = (sizeof(T) == 4 && NF == 1 && THREADS <= 256) ? 2 : 1;
  static constexpr int SMEM = (DPAD + NEL * 3 * NF * NP) * (int)sizeof(T) +
                              (TRI ? (NEL * 24 + 2 * NQ) * 4 : 0);
};

// geometry of node (i,j,k) of an element from its trilinear coefficients
// c[comp*8 + a], basis a = {1, r, s, t, rs, rt, st, rst}.
__device__ __forceinline__ void trilinear_G(const float* c, float r, float s, float t, float wijk,
                                            float& GwJ, float& G00, float& G01, float& G02,
                                            float& G11, float& G12, float& G22)
{
  float d[3][3];  // d[comp][dir]: x_r, x_s, x_t ...
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    const float* a = c + comp * 8;
    d[comp][0] = a[1] + a[4] * s + a[5] * t + a[7] * (s * t);
    d[comp][1] = a[2] + a[4] * r + a[6] * t + a[7] * (r * t);
    d[comp][2] = a[3] + a[5] * r + a[6] * s + a[7] * (r * s);
  }
  const float xr = d[0][0], xs = d[0][1], xt = d[0][2];
  const float yr = d[1][0], ys = d[1][1], yt = d[1][2];
  const float zr = d[2][0], zs = d[2][1], zt = d[2][2];
  // cofactor rows: J * grad r, J * grad s, J * grad t
  const float a0 = ys * zt - zs * yt, a1 = -(xs * zt - zs * xt), a2 = xs * yt - ys * xt;
  const float b0 = -(yr * zt - zr * yt), b1 = xr * zt - zr * xt, b2 = -(xr * yt - yr * xt);
  const float c0 = yr * zs - zr * ys, c1 = -(xr * zs - zr * xs), c2 = xr * ys - yr * xs;
  const float J = xr * a0 + yr * a1 + zr * a2;
  const float winv = __fdividef(wijk, J);  // J > 0 and O(h^3): the fast divide is exact enough
  GwJ = J * wijk;
  G00 = winv * (a0 * a0 + a1 * a1 + a2 * a2);
  G01 = winv * (a0 * b0 + a1 * b1 + a2 * b2);
  G02 = winv * (a0 * c0 + a1 * c1 + a2 * c2);
  G11 = winv * (b0 * b0 + b1 * b1 + b2 * b2);
  G12 = winv * (b0 * c0 + b1 * c1 + b2 * c2);
  G22 = winv * (c0 * c0 + c1 * c1 + c2 * c2);
}

template <int NQ, int NF, bool BK, bool PARTIAL, int PREC>
__global__ void __launch_bounds__(Cfg<NQ, NF, PREC>::THREADS, Cfg<NQ, NF, PREC>::MINB)
k_axhelm(const AxArgs a)
{
  using C = Cfg<NQ, NF, PREC>;
  using T = typename Prec<PREC>::T;
  using TG = typename Prec<PREC>::TG;
  constexpr int NQ2 = C::NQ2, NP = C::NP, NEL = C::NEL, DS = NQ + 1;
  if (a.skip != nullptr && *a.skip != 0) return;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_D = reinterpret_cast<T*>(smem_raw);
  T* s_all = s_D + C::DPAD;
  float* s_coef = reinterpret_cast<float*>(s_all + NEL * 3 * NF * NP);
  float* s_r = s_coef + NEL * 24;
  float* s_w = s_r + NQ;

  const int tid = threadIdx.x;
  const int el = tid / NQ2;
  const int ij = tid - el * NQ2;
  const int i = ij % NQ;
  const int j = ij / NQ;
  const int64_t eidx = (int64_t)blockIdx.x * NEL + el;
  const bool active = (el < NEL) && (eidx < a.Nelements);
  int64_t element = eidx;
  if (PARTIAL && active) element = a.elementList[eidx];

  const T* Dg = static_cast<const T*>(a.D);
  for (int t = tid; t < NQ2; t += blockDim.x) s_D[(t / NQ) * DS + (t % NQ)] = Dg[t];
  if (C::TRI) {
    const float* coef = static_cast<const float*>(a.ggeo);
    for (int t = tid; t < NEL * 24; t += blockDim.x) {
      const int e2 = t / 24;
      const int64_t ee = (int64_t)blockIdx.x * NEL + e2;
      if (ee < a.Nelements) {
        const int64_t elem = PARTIAL ? (int64_t)a.elementList[ee] : ee;
        s_coef[t] = coef[elem * 24 + (t - e2 * 24)];
      }
    }
    for (int t = tid; t < NQ; t += blockDim.x) {
      s_r[t] = a.r1d[t];
      s_w[t] = a.w1d[t];
    }
  }

  const int elc = active ? el : 0;  // keep shared pointers in range for idle threads
  T* s_q = s_all + elc * 3 * NF * NP;
  T* s_Gr = s_q + NF * NP;
  T* s_Gs = s_Gr + NF * NP;

  const TG* ge = static_cast<const TG*>(a.ggeo) + element * 7 * NP + ij;
  const TG* lam = static_cast<const TG*>(a.lambda);
  // 4-byte arithmetic with stored geometry is HBM-bound: the whole column's
  // geometric factors and lambdas are requested before the first barrier so
  // that every load of the element is in flight at once
  constexpr bool PF = (sizeof(T) == 4) && !C::TRI;  // stored geometry
  constexpr bool PFL = (sizeof(T) == 4) && !BK;     // lambda (also with trilinear geometry)
  constexpr int NPF = PF ? NQ : 1;
  TG pG[6][NPF];
  TG pW[PF && !BK ? NQ : 1], pL0[PFL ? NQ : 1], pL1[PFL ? NQ : 1];
  if ((PF || PFL) && active) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      if constexpr (PF) {
#pragma unroll
        for (int sl = 0; sl < 6; ++sl) pG[sl][k] = ge[(sl + 1) * NP + k * NQ2];
      }
      if constexpr (PF && !BK) pW[k] = ge[k * NQ2];
      if constexpr (PFL) {
        pL0[k] = lam[element * NP + k * NQ2 + ij];
        pL1[k] = lam[element * NP + k * NQ2 + ij + a.offset];
      }
    }
  }

  T r_q[NF][NQ];
  if (active) {
    const T* qe = static_cast<const T*>(a.q) + element * NP + ij;
#pragma unroll
    for (int f = 0; f < NF; ++f)
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const T v = qe[f * a.offset + k * NQ2];
        r_q[f][k] = v;
        s_q[f * NP + k * NQ2 + ij] = v;
      }
  }
  __syncthreads();

  T r_Gt[NF][NQ];
  float r_gw[C::TRI && !BK ? NQ : 1];  // GwJ of the column, trilinear geometry only
  if (active) {
    float rr = 0.f, ss = 0.f, wij = 0.f;
    if (C::TRI) {
      rr = s_r[i];
      ss = s_r[j];
      wij = s_w[i] * s_w[j];
    }
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const int n = k * NQ2 + ij;
      T G00, G01, G02, G11, G12, G22;
      if (C::TRI) {
        float gw, g00, g01, g02, g11, g12, g22;
        trilinear_G(s_coef + elc * 24, rr, ss, s_r[k], wij * s_w[k], gw, g00, g01, g02, g11, g12,
                    g22);
        G00 = g00; G01 = g01; G02 = g02; G11 = g11; G12 = g12; G22 = g22;
        if constexpr (C::TRI && !BK) r_gw[k] = gw;
      } else if constexpr (PF) {
        G00 = to_c(pG[0][k]);
        G01 = to_c(pG[1][k]);
        G02 = to_c(pG[2][k]);
        G11 = to_c(pG[3][k]);
        G12 = to_c(pG[4][k]);
        G22 = to_c(pG[5][k]);
      } else {
        G00 = to_c(ge[1 * NP + k * NQ2]);
        G01 = to_c(ge[2 * NP + k * NQ2]);
        G02 = to_c(ge[3 * NP + k * NQ2]);
        G11 = to_c(ge[4 * NP + k * NQ2]);
        G12 = to_c(ge[5 * NP + k * NQ2]);
        G22 = to_c(ge[6 * NP + k * NQ2]);
      }
      T lam0 = T(1);
      if constexpr (!BK && PFL) {
        lam0 = to_c(pL0[k]);
      } else if constexpr (!BK) {
        lam0 = to_c(lam[element * NP + n]);
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const T* sq = s_q + f * NP + k * NQ2;
        T qr = 0, qs = 0, qt = 0;
#pragma unroll
        for (int m = 0; m < NQ; ++m) {
          qr += s_D[i * DS + m] * sq[j * NQ + m];
          qs += s_D[j * DS + m] * sq[m * NQ + i];
          qt += s_D[k * DS + m] * r_q[f][m];
        }
        T gr = G00 * qr + G01 * qs + G02 * qt;
        T gs = G01 * qr + G11 * qs + G12 * qt;
        T gt = G02 * qr + G12 * qs + G22 * qt;
        if (!BK) {
          gr *= lam0;
          gs *= lam0;
          gt *= lam0;
        }
        s_Gr[f * NP + n] = gr;
        s_Gs[f * NP + n] = gs;
        r_Gt[f][k] = gt;
      }
    }
  }
  __syncthreads();

  T qaq = T(0);  // this thread's share of q . Aq (when asked for)
  if (active) {
    T* Aqe = static_cast<T*>(a.Aq) + element * NP + ij;
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const int n = k * NQ2 + ij;
      T wl1 = T(0);
      if (!BK) {
        T GwJ, lam1;
        if constexpr (C::TRI && !BK) {
          GwJ = r_gw[k];
          lam1 = to_c(pL1[k]);
        } else if constexpr (PF && !BK) {
          GwJ = to_c(pW[k]);
          lam1 = to_c(pL1[k]);
        } else {
          GwJ = to_c(ge[k * NQ2]);
          lam1 = to_c(lam[element * NP + n + a.offset]);
        }
        wl1 = GwJ * lam1;
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const T* gr = s_Gr + f * NP + k * NQ2;
        const T* gs = s_Gs + f * NP + k * NQ2;
        T ar = 0, as = 0, at = 0;
#pragma unroll
        for (int m = 0; m < NQ; ++m) {
          ar += s_D[m * DS + i] * gr[j * NQ + m];
          as += s_D[m * DS + j] * gs[m * NQ + i];
          at += s_D[m * DS + k] * r_Gt[f][m];
        }
        T out = ar + as + at;
        if (!BK) out += wl1 * r_q[f][k];
        Aqe[f * a.offset + k * NQ2] = out;
        qaq += r_q[f][k] * out;
      }
    }
  }
  if (!PARTIAL && a.dot_partials != nullptr) {  // block sum in a fixed order
    __shared__ double s_red[32];
    double v = (double)qaq;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) s_red[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_red[w];
      a.dot_partials[blockIdx.x] = t;
      if (blockIdx.x == 0) *a.dot_count = (int)gridDim.x;
    }
  }
}

template <int NQ, int NF, bool BK, bool PARTIAL, int PREC>
int run(const AxArgs& a, cudaStream_t s)
{
  using C = Cfg<NQ, NF, PREC>;
  auto kern = k_axhelm<NQ, NF, BK, PARTIAL, PREC>;
  // opt in to >48 KB of shared memory at the first launch on each device
  static SmemOptIn smem_opt;
  NEKB_TRY(smem_opt.ensure(kern, C::SMEM));  // dynamic + static may pass 48 KB
  const int64_t nblk = (a.Nelements + C::NEL - 1) / C::NEL;
  if (nblk == 0) return NEKB_OK;
  if (nblk > INT_MAX) return fail(NEKB_ERR_INVALID, "axhelm: too many elements");
  kern<<<(unsigned)nblk, C::THREADS, C::SMEM, s>>>(a);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

// all variants of one order and precision; Partial forms are built for FP64 only
template <int NQ, int PREC>
int run_flags(int flags, const AxArgs& a, cudaStream_t s)
{
  const bool bk = flags & NEKB_AX_BK, n3 = flags & NEKB_AX_N3, part = flags & NEKB_AX_PARTIAL;
  if (part) {
    if constexpr (PREC == NEKB_FP64) {
      if (n3) return bk ? run<NQ, 3, true, true, PREC>(a, s) : run<NQ, 3, false, true, PREC>(a, s);
      return bk ? run<NQ, 1, true, true, PREC>(a, s) : run<NQ, 1, false, true, PREC>(a, s);
    } else {
      return fail(NEKB_ERR_UNSUPPORTED, "axhelm: Partial variants are built for FP64 only");
    }
  }
  if (n3) return bk ? run<NQ, 3, true, false, PREC>(a, s) : run<NQ, 3, false, false, PREC>(a, s);
  return bk ? run<NQ, 1, true, false, PREC>(a, s) : run<NQ, 1, false, false, PREC>(a, s);
}

}  // namespace ax
}  // namespace nekb
