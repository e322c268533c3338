// FP64 axhelm with the even-odd form of the tensor-product contractions.
//
// GB300 executes FP64 at about two fused multiply-adds per clock per SM, so
// the FP64 operator is bound by its FP64 instruction count (at N=7 its HBM
// time is a ninth of its FP64 time).  This kernel issues as few FP64
// operations per node as the operator's structure allows; shared memory,
// integer work and barriers are cheap next to the FP64 pipe.
//
// For nodes symmetric about the element centre (GLL or Gauss) the 1D
// derivative matrix is centro-antisymmetric, D[NQ-1-p][NQ-1-m] = -D[p][m].
// Split a line of values v into even and odd parts, e_m = v_m + v_m',
// o_m = v_m - v_m' (m' = NQ-1-m, m < H = NQ/2; the middle value e_H = v_H when
// NQ is odd).  Then, for p < H,
//   (D v)_p  = s_p + d_p,   (D v)_p' = s_p - d_p,
//   s_p = sum_{m<H} (D[p][m] + D[p'][m])/2 o_m,
//   d_p = sum_{m<H} (D[p][m] - D[p'][m])/2 e_m  (+ D[p][H] e_H, NQ odd),
// and the middle output (NQ odd) is sum_{m<H} D[H][m] o_m.  A line of NQ
// outputs costs about NQ/2 + 2 FP64 operations per output instead of NQ; D^T
// (the second set of contractions) has the same structure.  At N=7 the BK
// operator drops from 59 to 47 FP64 operations per node.
//
// Mapping: as in the direct kernel, thread (i,j) of an element owns the
// k-column of nodes (i,j,0..NQ-1), so the t direction runs in registers.  The
// r and s directions go through shared memory: every thread writes the
// even/odd values of its own nodes (its partner's q it reads from global
// memory, so the first transform needs no barrier), then evaluates "pair
// tasks": both outputs of one pair p of one line.  Thread i of line j takes
// tasks i*T .. i*T+T-1 of that line's (pair, plane) list, with T = H (NQ even)
// or H+1 (NQ odd, where the middle output is a pair task whose d-row is zero
// and whose two outputs land on the same node).  Every thread of a warp runs
// the same FP64 instruction stream: a divergent FP64 instruction would occupy
// the pipe as long as a full one.  Five barriers per element and field.
//
// Callers may pass any D.  Each CTA checks D for centro-antisymmetry
// (|D[p][m] + D[p'][m']| <= 2^-46 max|D|); when it does not hold the CTA
// evaluates the direct sums instead, so no result depends on the property.
#pragma once

#include "internal.h"

#include <climits>

namespace nekb {
namespace ax_eo {

template <int NQ>
struct CfgEO {
  static constexpr int H = NQ / 2;
  static constexpr int ODD = NQ & 1;
  static constexpr int HM = H + ODD;       // even part, with the middle value when NQ is odd
  static constexpr int HP = H + ODD;       // pair tasks per line (incl. the middle line)
  static constexpr int NQ2 = NQ * NQ;
  static constexpr int NP = NQ2 * NQ;
  static constexpr int PER_EL = 4 * NP * 8;  // four node arrays per element, fields in turn
  static constexpr int CAP = 100 * 1024;     // two CTAs per SM
  static constexpr int nel_fit(int n) { return (n <= 1 || n * PER_EL <= CAP) ? n : nel_fit(n - 1); }
  static constexpr int NEL0 = (256 / NQ2) > 0 ? (256 / NQ2) : 1;
  static constexpr int NEL = nel_fit(NEL0);
  static constexpr int THREADS = ((NEL * NQ2 + 31) / 32) * 32;
  static constexpr int DS = NQ + 1;  // row stride of D in shared memory
  static constexpr int DPAD = ((NQ * DS) + 1) & ~1;
  // per matrix (D, then D^T): P[HP][H] (s rows; row H = middle row, NQ odd)
  // and M[HP][HM] (d rows; row H is zero)
  static constexpr int TAB = HP * H + HP * HM;
  static constexpr int SMEM = (DPAD + 2 * TAB + NEL * 4 * NP) * 8;
};

// transformed value of node `pos` of a line from its own value and its
// partner's (pos' = NQ-1-pos): e at pos < pos', o at pos > pos', the value
// itself in the middle; one FP64 operation for every thread
__device__ __forceinline__ double eo_value(double own, double partner, int pos, int ppos)
{
  const double sg = pos > ppos ? -1.0 : 1.0;
  const double pv = pos == ppos ? 0.0 : partner;
  return fma(sg, own, pv);
}

// s and d of pair p from a transformed line (e_m at position m, o_m at
// position NQ-1-m, the middle value at position H), elements `stride` apart
template <int NQ>
__device__ __forceinline__ void pair_sd(const double* line, int stride, const double* P,
                                        const double* M, double& s, double& d)
{
  using C = CfgEO<NQ>;
  constexpr int H = C::H, HM = C::HM;
  s = P[0] * line[(NQ - 1) * stride];
#pragma unroll
  for (int m = 1; m < H; ++m) s = fma(P[m], line[(NQ - 1 - m) * stride], s);
  d = M[0] * line[0];
#pragma unroll
  for (int m = 1; m < HM; ++m) d = fma(M[m], line[m * stride], d);
}

// all NQ outputs of a line held in registers
template <int NQ>
__device__ __forceinline__ void line_eo(const double (&v)[NQ], double (&out)[NQ], const double* P,
                                        const double* M)
{
  using C = CfgEO<NQ>;
  constexpr int H = C::H, HM = C::HM;
  double e[HM], o[H];
#pragma unroll
  for (int m = 0; m < H; ++m) {
    e[m] = v[m] + v[NQ - 1 - m];
    o[m] = v[m] - v[NQ - 1 - m];
  }
  if constexpr (C::ODD) e[H] = v[H];
#pragma unroll
  for (int p = 0; p < H; ++p) {
    double s = P[p * H] * o[0];
#pragma unroll
    for (int m = 1; m < H; ++m) s = fma(P[p * H + m], o[m], s);
    double d = M[p * HM] * e[0];
#pragma unroll
    for (int m = 1; m < HM; ++m) d = fma(M[p * HM + m], e[m], d);
    out[p] = s + d;
    out[NQ - 1 - p] = s - d;
  }
  if constexpr (C::ODD) {
    double s = P[H * H] * o[0];
#pragma unroll
    for (int m = 1; m < H; ++m) s = fma(P[H * H + m], o[m], s);
    out[H] = s;
  }
}

// pair tasks of the r direction (lines along i, nodes 1 apart) or the s
// direction (lines along j, nodes NQ apart) for thread (a, b): a is the
// thread's index along the line direction, b its index across
template <int NQ, bool RDIR>
__device__ __forceinline__ void pair_tasks(const double* T, double* Q, int a, int b,
                                           const double* P, const double* M)
{
  using C = CfgEO<NQ>;
  constexpr int H = C::H, HM = C::HM, HP = C::HP, NQ2 = C::NQ2;
  constexpr int stride = RDIR ? 1 : NQ;
  const int cross = RDIR ? b * NQ : b;  // offset of the line inside its plane
#pragma unroll
  for (int t = 0; t < HP; ++t) {
    const int tau = a * HP + t;  // (pair, plane) task index of this line
    const int p = tau / NQ, k = tau - p * NQ;
    const double* line = T + k * NQ2 + cross;
    double s, d;
    pair_sd<NQ>(line, stride, P + p * H, M + p * HM, s, d);
    double* out = Q + k * NQ2 + cross;
    out[p * stride] = s + d;
    out[(NQ - 1 - p) * stride] = s - d;  // the same node and value for the middle line
  }
}

// the direct sums, for a D that is not centro-antisymmetric: q in A0, Gr in A1,
// Gs in A2 (the FP64 path of the direct kernel)
template <int NQ, bool BK>
__device__ __forceinline__ void direct_field(const AxArgs& a, int f, int64_t element, int ij,
                                             int i, int j, bool active, const double* s_D,
                                             double* A0, double* A1, double* A2, double& qaq)
{
  using C = CfgEO<NQ>;
  constexpr int NQ2 = C::NQ2, NP = C::NP, DS = C::DS;
  const double* ge = static_cast<const double*>(a.ggeo) + element * 7 * NP + ij;
  const double* lam = static_cast<const double*>(a.lambda);
  double r_q[NQ], r_Gt[NQ];
  if (active) {
    const double* qe = static_cast<const double*>(a.q) + f * a.offset + element * NP + ij;
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      r_q[k] = qe[k * NQ2];
      A0[k * NQ2 + ij] = r_q[k];
    }
  }
  __syncthreads();
  if (active) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const int n = k * NQ2 + ij;
      double qr = 0, qs = 0, qt = 0;
#pragma unroll
      for (int m = 0; m < NQ; ++m) {
        qr += s_D[i * DS + m] * A0[k * NQ2 + j * NQ + m];
        qs += s_D[j * DS + m] * A0[k * NQ2 + m * NQ + i];
        qt += s_D[k * DS + m] * r_q[m];
      }
      const double G00 = ge[1 * NP + k * NQ2], G01 = ge[2 * NP + k * NQ2];
      const double G02 = ge[3 * NP + k * NQ2], G11 = ge[4 * NP + k * NQ2];
      const double G12 = ge[5 * NP + k * NQ2], G22 = ge[6 * NP + k * NQ2];
      double gr = G00 * qr + G01 * qs + G02 * qt;
      double gs = G01 * qr + G11 * qs + G12 * qt;
      double gt = G02 * qr + G12 * qs + G22 * qt;
      if (!BK) {
        const double lam0 = lam[element * NP + n];
        gr *= lam0;
        gs *= lam0;
        gt *= lam0;
      }
      A1[n] = gr;
      A2[n] = gs;
      r_Gt[k] = gt;
    }
  }
  __syncthreads();
  if (active) {
    double* Aqe = static_cast<double*>(a.Aq) + f * a.offset + element * NP + ij;
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      double ar = 0, as = 0, at = 0;
#pragma unroll
      for (int m = 0; m < NQ; ++m) {
        ar += s_D[m * DS + i] * A1[k * NQ2 + j * NQ + m];
        as += s_D[m * DS + j] * A2[k * NQ2 + m * NQ + i];
        at += s_D[m * DS + k] * r_Gt[m];
      }
      double out = ar + as + at;
      if (!BK) out += (ge[k * NQ2] * lam[element * NP + k * NQ2 + ij + a.offset]) * r_q[k];
      Aqe[k * NQ2] = out;
      qaq += r_q[k] * out;
    }
  }
  __syncthreads();  // the next field overwrites A0..A2
}

template <int NQ, int NF, bool BK, bool PARTIAL>
__global__ void __launch_bounds__(CfgEO<NQ>::THREADS, 2) k_axhelm_eo(const AxArgs a)
{
  using C = CfgEO<NQ>;
  constexpr int H = C::H, HM = C::HM, HP = C::HP, NQ2 = C::NQ2, NP = C::NP, NEL = C::NEL;
  constexpr int DS = C::DS;
  if (a.skip != nullptr && *a.skip != 0) return;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* s_D = reinterpret_cast<double*>(smem_raw);
  double* s_P1 = s_D + C::DPAD;  // D
  double* s_M1 = s_P1 + HP * H;
  double* s_P2 = s_M1 + HP * HM;  // D^T
  double* s_M2 = s_P2 + HP * H;
  double* s_all = s_M2 + HP * HM;
  __shared__ int s_sym;

  const int tid = threadIdx.x;
  const double* Dg = static_cast<const double*>(a.D);
  for (int t = tid; t < NQ2; t += blockDim.x) s_D[(t / NQ) * DS + (t % NQ)] = Dg[t];
  __syncthreads();
  if (tid < 32) {  // is D centro-antisymmetric?
    double mx = 0.0, asym = 0.0;
    for (int t = tid; t < NQ2; t += 32) {
      const int r = t / NQ, c = t - (t / NQ) * NQ;
      const double v = s_D[r * DS + c];
      mx = fmax(mx, fabs(v));
      asym = fmax(asym, fabs(v + s_D[(NQ - 1 - r) * DS + (NQ - 1 - c)]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      asym = fmax(asym, __shfl_xor_sync(0xffffffffu, asym, o));
    }
    if (tid == 0) s_sym = (asym <= 0x1p-46 * mx) ? 1 : 0;
  }
  // coefficient rows with the halves folded in; D^T[p][m] = D[m][p]
  for (int t = tid; t < HP * HM; t += blockDim.x) {
    const int p = t / HM, m = t - (t / HM) * HM, pp = NQ - 1 - p;
    if (p < H) {
      if (m < H) {
        s_P1[p * H + m] = 0.5 * (s_D[p * DS + m] + s_D[pp * DS + m]);
        s_M1[p * HM + m] = 0.5 * (s_D[p * DS + m] - s_D[pp * DS + m]);
        s_P2[p * H + m] = 0.5 * (s_D[m * DS + p] + s_D[m * DS + pp]);
        s_M2[p * HM + m] = 0.5 * (s_D[m * DS + p] - s_D[m * DS + pp]);
      } else {  // middle column, NQ odd
        s_M1[p * HM + m] = s_D[p * DS + H];
        s_M2[p * HM + m] = s_D[H * DS + p];
      }
    } else {  // middle row, NQ odd: s = sum D[H][m] o_m, d = 0
      if (m < H) {
        s_P1[H * H + m] = s_D[H * DS + m];
        s_P2[H * H + m] = s_D[m * DS + H];
      }
      s_M1[H * HM + m] = 0.0;
      s_M2[H * HM + m] = 0.0;
    }
  }
  __syncthreads();
  const bool sym = s_sym != 0;  // the same for every thread of the CTA

  const int el = tid / NQ2;
  const int ij = tid - el * NQ2;
  const int i = ij % NQ;
  const int j = ij / NQ;
  const int ip = NQ - 1 - i, jp = NQ - 1 - j;
  const int64_t eidx = (int64_t)blockIdx.x * NEL + el;
  const bool active = (el < NEL) && (eidx < a.Nelements);
  int64_t element = eidx;
  if (PARTIAL && active) element = a.elementList[eidx];
  const int elc = active ? el : 0;  // keep shared pointers in range for idle threads
  double* A0 = s_all + elc * 4 * NP;
  double* A1 = A0 + NP;
  double* A2 = A1 + NP;
  double* A3 = A2 + NP;

  const double* ge = static_cast<const double*>(a.ggeo) + element * 7 * NP + ij;
  const double* lam = static_cast<const double*>(a.lambda);
  double qaq = 0.0;  // this thread's share of q . Aq (when asked for)

#pragma unroll 1
  for (int f = 0; f < NF; ++f) {
    if (!sym) {
      direct_field<NQ, BK>(a, f, element, ij, i, j, active, s_D, A0, A1, A2, qaq);
      continue;
    }
    if (f > 0) __syncthreads();  // the previous field's last reads of A0, A1
    double r_q[NQ], qt[NQ];
    if (active) {
      const double* qe = static_cast<const double*>(a.q) + f * a.offset + element * NP + ij;
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const double v = qe[k * NQ2];
        const double vi = qe[k * NQ2 + (ip - i)];
        const double vj = qe[k * NQ2 + (jp - j) * NQ];
        r_q[k] = v;
        A0[k * NQ2 + ij] = eo_value(v, vi, i, ip);
        A1[k * NQ2 + ij] = eo_value(v, vj, j, jp);
      }
      line_eo<NQ>(r_q, qt, s_P1, s_M1);  // t direction
    }
    __syncthreads();
    if (active) {
      pair_tasks<NQ, true>(A0, A2, i, j, s_P1, s_M1);   // qr
      pair_tasks<NQ, false>(A1, A3, j, i, s_P1, s_M1);  // qs
    }
    __syncthreads();
    double gt[NQ];
    if (active) {
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const int n = k * NQ2 + ij;
        const double qr = A2[n], qs = A3[n];
        const double G00 = ge[1 * NP + k * NQ2], G01 = ge[2 * NP + k * NQ2];
        const double G02 = ge[3 * NP + k * NQ2], G11 = ge[4 * NP + k * NQ2];
        const double G12 = ge[5 * NP + k * NQ2], G22 = ge[6 * NP + k * NQ2];
        double gr = G00 * qr + G01 * qs + G02 * qt[k];
        double gs = G01 * qr + G11 * qs + G12 * qt[k];
        double g3 = G02 * qr + G12 * qs + G22 * qt[k];
        if (!BK) {
          const double lam0 = lam[element * NP + n];
          gr *= lam0;
          gs *= lam0;
          g3 *= lam0;
        }
        A0[n] = gr;
        A1[n] = gs;
        gt[k] = g3;
      }
    }
    __syncthreads();
    double at[NQ];
    if (active) {
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const int n = k * NQ2 + ij;
        A2[n] = eo_value(A0[n], A0[n + (ip - i)], i, ip);
        A3[n] = eo_value(A1[n], A1[n + (jp - j) * NQ], j, jp);
      }
      line_eo<NQ>(gt, at, s_P2, s_M2);  // t direction, D^T
    }
    __syncthreads();
    if (active) {
      pair_tasks<NQ, true>(A2, A0, i, j, s_P2, s_M2);   // r part of Aq
      pair_tasks<NQ, false>(A3, A1, j, i, s_P2, s_M2);  // s part of Aq
    }
    __syncthreads();
    if (active) {
      double* Aqe = static_cast<double*>(a.Aq) + f * a.offset + element * NP + ij;
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const int n = k * NQ2 + ij;
        double out = A0[n] + A1[n] + at[k];
        if (!BK) out += (ge[k * NQ2] * lam[element * NP + n + a.offset]) * r_q[k];
        Aqe[k * NQ2] = out;
        qaq += r_q[k] * out;
      }
    }
  }
  if (!PARTIAL && a.dot_partials != nullptr) {  // block sum in a fixed order
    __shared__ double s_red[32];
    double v = qaq;
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

template <int NQ, int NF, bool BK, bool PARTIAL>
int run(const AxArgs& a, cudaStream_t s)
{
  using C = CfgEO<NQ>;
  static_assert(C::SMEM <= 227 * 1024, "even-odd axhelm: shared memory plan exceeds 227 KB");
  auto kern = k_axhelm_eo<NQ, NF, BK, PARTIAL>;
  static SmemOptIn smem_opt;
  NEKB_TRY(smem_opt.ensure(kern, C::SMEM));  // dynamic + static may pass 48 KB
  const int64_t nblk = (a.Nelements + C::NEL - 1) / C::NEL;
  if (nblk == 0) return NEKB_OK;
  if (nblk > INT_MAX) return fail(NEKB_ERR_INVALID, "axhelm: too many elements");
  kern<<<(unsigned)nblk, C::THREADS, C::SMEM, s>>>(a);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

// all FP64 variants of one order (Partial forms included)
template <int NQ>
int run_flags(int flags, const AxArgs& a, cudaStream_t s)
{
  const bool bk = flags & NEKB_AX_BK, n3 = flags & NEKB_AX_N3, part = flags & NEKB_AX_PARTIAL;
  if (part) {
    if (n3) return bk ? run<NQ, 3, true, true>(a, s) : run<NQ, 3, false, true>(a, s);
    return bk ? run<NQ, 1, true, true>(a, s) : run<NQ, 1, false, true>(a, s);
  }
  if (n3) return bk ? run<NQ, 3, true, false>(a, s) : run<NQ, 3, false, false>(a, s);
  return bk ? run<NQ, 1, true, false>(a, s) : run<NQ, 1, false, false>(a, s);
}

}  // namespace ax_eo
}  // namespace nekb
