// Learned element preconditioner: a 3-layer 3x3x3 convolution network on the
// Nq^3 nodes of each element (channels 1 -> C -> C -> 1, tanh-form GELU after
// the first two layers, zero padding at the element boundary, no bias).
//
// Kernels (one CTA per element at a time, one thread per node, all
// activations in shared memory):
//   k_net_infer : BF16 weights (FP32 in shared memory), FP32 accumulation;
//                 input normalised by the element RMS and the output scaled
//                 back, so the map is positively homogeneous in r_e.
//   k_net_train : forward, loss, backward-data and weight gradients of a batch
//                 of elements fused in one kernel; per-block partial gradients.
//   k_net_reduce: fixed-order sum of the partials (deterministic), then Adam.
// In the solver: z = invDiag*r + mask(gs(w * h * s_e * net(h r_e / s_e))),
// h = sqrt(invDiag) per node, s_e = RMS of h r over element e.
// No counterpart in the reference.
#include "nn.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

struct nekb_net {
  int Nq = 0, Np = 0, C = 0, P = 0;
  int64_t step = 0;
  float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  nekb::DeviceBuf W, Wbf, m, v, grad, gpart, lpart, loss;
  int gblocks = 0;
  int inference = NEKB_NET_TENSOR;  // NEKB_NET_TENSOR where built (Nq=8, C=16), else FP32 cores
};

namespace nekb {
namespace {

constexpr int kTaps = 27;

__host__ __device__ constexpr int np_of(int nq) { return nq * nq * nq; }
__host__ __device__ constexpr int nparams(int c) { return kTaps * c * (c + 2); }
__host__ __device__ constexpr int threads_of(int nq) { return ((np_of(nq) + 31) / 32) * 32; }

__device__ __forceinline__ float gelu(float x)
{
  const float c = 0.7978845608028654f;
  return 0.5f * x * (1.0f + tanhf(c * (x + 0.044715f * x * x * x)));
}

__device__ __forceinline__ float gelu_grad(float x)
{
  const float c = 0.7978845608028654f;
  const float t = tanhf(c * (x + 0.044715f * x * x * x));
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * c * (1.0f + 3.0f * 0.044715f * x * x);
}

// tap t = (di+1) + 3(dj+1) + 9(dk+1); neighbour offset in the element
template <int NQ>
__device__ __forceinline__ int tap_off(int t)
{
  const int di = t % 3 - 1, dj = (t / 3) % 3 - 1, dk = t / 9 - 1;
  return di + NQ * dj + NQ * NQ * dk;
}

// bit t set when node (i,j,k) + tap t lies inside the element
template <int NQ>
__device__ __forceinline__ unsigned tap_mask(int i, int j, int k)
{
  unsigned m = 0;
#pragma unroll
  for (int t = 0; t < kTaps; ++t) {
    const int di = t % 3 - 1, dj = (t / 3) % 3 - 1, dk = t / 9 - 1;
    const int a = i + di, b = j + dj, c = k + dk;
    if (a >= 0 && a < NQ && b >= 0 && b < NQ && c >= 0 && c < NQ) m |= 1u << t;
  }
  return m;
}

__device__ __forceinline__ float block_sum_f(float v, float* red)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  float s = 0.f;
  const int nw = blockDim.x >> 5;
  for (int w = 0; w < nw; ++w) s += red[w];  // every thread, fixed order
  return s;
}

// forward conv with C_OUT outputs for node n; weights in shared memory as
// [ci][tap][co] (co fastest)
template <int NQ, int CIN, int COUT>
__device__ __forceinline__ void conv_fwd(const float* in, const float* w, int n, unsigned msk,
                                         float (&acc)[COUT])
{
  constexpr int NP = np_of(NQ);
#pragma unroll
  for (int co = 0; co < COUT; ++co) acc[co] = 0.f;
#pragma unroll 1
  for (int ci = 0; ci < CIN; ++ci) {
    const float* src = in + ci * NP + n;
#pragma unroll
    for (int t = 0; t < kTaps; ++t) {
      if (!(msk & (1u << t))) continue;
      const float x = src[tap_off<NQ>(t)];
      const float* wt = w + (ci * kTaps + t) * COUT;
      if constexpr (COUT % 4 == 0) {
        // the COUT weights of one (ci, tap) are contiguous and 16-byte aligned
        const float4* w4 = reinterpret_cast<const float4*>(wt);
#pragma unroll
        for (int q = 0; q < COUT / 4; ++q) {
          const float4 v = w4[q];
          acc[4 * q + 0] += v.x * x;
          acc[4 * q + 1] += v.y * x;
          acc[4 * q + 2] += v.z * x;
          acc[4 * q + 3] += v.w * x;
        }
      } else {
#pragma unroll
        for (int co = 0; co < COUT; ++co) acc[co] += wt[co] * x;
      }
    }
  }
}

// weights [co][ci][t] (global, FP32 or BF16) -> shared [ci][t][co] FP32
template <typename TW>
__device__ void load_weights(const TW* W, float* sW, int C)
{
  const int o2 = kTaps * C, o3 = kTaps * C + kTaps * C * C, P = nparams(C);
  for (int p = threadIdx.x; p < P; p += blockDim.x) {
    float val;
    if constexpr (sizeof(TW) == 2)
      val = __bfloat162float(W[p]);
    else
      val = W[p];
    int dst;
    if (p < o2) {  // layer 1: [co][0][t] -> [0][t][co]
      const int co = p / kTaps, t = p % kTaps;
      dst = t * C + co;
    } else if (p < o3) {  // layer 2: [co][ci][t] -> [ci][t][co]
      const int q = p - o2, co = q / (C * kTaps), ci = (q / kTaps) % C, t = q % kTaps;
      dst = o2 + (ci * kTaps + t) * C + co;
    } else {  // layer 3: [0][ci][t] -> [ci][t][0]
      dst = p;
    }
    sW[dst] = val;
  }
}

// mode bit kNetNormalize: input h r_e / s_e with h = sqrt(invDiag) per node (1
// without invDiag) and s_e = RMS of h r_e; output times w * h * s_e.  Bit
// kNetAddJacobi: w * invDiag * r is added to the output, so that a gather-
// scatter of it yields invDiag r + gs(w h s net) (invDiag and r are continuous
// across element copies and the weights w of a group sum to one).  The symmetric
// diagonal scaling makes the map the network has to represent nearly uniform
// across the GLL nodes (whose weights span three decades at N=7) and
// independent of the element size.
template <int NQ, int C>
__global__ void __launch_bounds__(threads_of(NQ))
k_net_infer(int64_t Etot, int64_t Efield, const __nv_bfloat16* __restrict__ Wbf,
            const float* __restrict__ r, const float* __restrict__ w,
            const float* __restrict__ invDiag, float* __restrict__ out, int normalize,
            const int* skip)
{
  if (skip != nullptr && *skip != 0) return;
  constexpr int NP = np_of(NQ), P = nparams(C), o2 = kTaps * C, o3 = kTaps * C + kTaps * C * C;
  extern __shared__ __align__(16) float sm[];
  float* sW = sm;
  float* a0 = sW + P;
  float* a1 = a0 + NP;
  float* a2 = a1 + C * NP;
  __shared__ float red[32];
  load_weights(Wbf, sW, C);
  const int n = threadIdx.x;
  const bool act = n < NP;
  const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
  const unsigned msk = act ? tap_mask<NQ>(i, j, k) : 0u;
  for (int64_t e = blockIdx.x; e < Etot; e += gridDim.x) {
    const float h = (act && invDiag) ? sqrtf(invDiag[(e % Efield) * NP + n]) : 1.f;
    const float v = act ? h * r[e * NP + n] : 0.f;
    float s = 1.f;
    if (normalize & kNetNormalize) s = sqrtf(block_sum_f(v * v, red) / NP);
    const float inv = s > 0.f ? 1.f / s : 0.f;
    if (act) a0[n] = v * inv;
    __syncthreads();
    if (act) {
      float acc[C];
      conv_fwd<NQ, 1, C>(a0, sW, n, msk, acc);
#pragma unroll
      for (int co = 0; co < C; ++co) a1[co * NP + n] = gelu(acc[co]);
    }
    __syncthreads();
    if (act) {
      float acc[C];
      conv_fwd<NQ, C, C>(a1, sW + o2, n, msk, acc);
#pragma unroll
      for (int co = 0; co < C; ++co) a2[co * NP + n] = gelu(acc[co]);
    }
    __syncthreads();
    if (act) {
      float acc[1];
      conv_fwd<NQ, C, 1>(a2, sW + o3, n, msk, acc);
      const float wn = w ? w[(e % Efield) * NP + n] : 1.f;
      float o = h * s * acc[0];
      if ((normalize & kNetAddJacobi) && invDiag) o += invDiag[(e % Efield) * NP + n] * r[e * NP + n];
      out[e * NP + n] = wn * o;
    }
    __syncthreads();
  }
}

// weight gradient of one layer for one element, accumulated into gW[co][ci][t]:
// gW += sum_n gout[co][n] * in[ci][n + off_t]
template <int NQ>
__device__ void accum_wgrad(const float* gout, const float* in, float* gW, int Cin, int Cout)
{
  constexpr int NP = np_of(NQ);
  const int total = Cout * Cin * kTaps;
  for (int p = threadIdx.x; p < total; p += blockDim.x) {
    const int co = p / (Cin * kTaps), ci = (p / kTaps) % Cin, t = p % kTaps;
    const int di = t % 3 - 1, dj = (t / 3) % 3 - 1, dk = t / 9 - 1;
    const int i0 = di < 0 ? 1 : 0, i1 = di > 0 ? NQ - 1 : NQ;
    const int j0 = dj < 0 ? 1 : 0, j1 = dj > 0 ? NQ - 1 : NQ;
    const int k0 = dk < 0 ? 1 : 0, k1 = dk > 0 ? NQ - 1 : NQ;
    const int off = di + NQ * dj + NQ * NQ * dk;
    const float* g = gout + co * NP;
    const float* x = in + ci * NP;
    float acc = 0.f;
    for (int kk = k0; kk < k1; ++kk)
      for (int jj = j0; jj < j1; ++jj)
        for (int ii = i0; ii < i1; ++ii) {
          const int nn = ii + NQ * (jj + NQ * kk);
          acc += g[nn] * x[nn + off];
        }
    gW[p] += acc;
  }
}

// backward-data: gin[ci][n] = sum_co sum_t W[co][ci][t] gout[co][n - off_t],
// weights in shared memory as [ci][t][co]; result times gelu'(z) when z != null
template <int NQ, int CIN, int COUT>
__device__ __forceinline__ void conv_bwd_data(const float* gout, const float* w, int n,
                                              unsigned msk_in, float (&acc)[CIN])
{
  constexpr int NP = np_of(NQ);
#pragma unroll
  for (int ci = 0; ci < CIN; ++ci) acc[ci] = 0.f;
#pragma unroll 1
  for (int co = 0; co < COUT; ++co) {
    const float* g = gout + co * NP + n;
#pragma unroll
    for (int t = 0; t < kTaps; ++t) {
      // output node o = n - off_t used n as its tap-t neighbour; o is inside
      // the element exactly when n + off_(26-t) is (the mirrored tap)
      if (!(msk_in & (1u << (kTaps - 1 - t)))) continue;
      const float gv = g[-tap_off<NQ>(t)];
#pragma unroll
      for (int ci = 0; ci < CIN; ++ci) acc[ci] += w[(ci * kTaps + t) * COUT + co] * gv;
    }
  }
}

template <int NQ, int C>
__global__ void __launch_bounds__(threads_of(NQ))
k_net_train(int64_t E, const float* __restrict__ W, const float* __restrict__ in,
            const float* __restrict__ target, float gscale, float* __restrict__ gpart,
            float* __restrict__ lpart)
{
  constexpr int NP = np_of(NQ), P = nparams(C), o2 = kTaps * C, o3 = kTaps * C + kTaps * C * C;
  extern __shared__ __align__(16) float sm[];
  float* sW = sm;        // P, [ci][t][co]
  float* gW = sW + P;    // P, [co][ci][t]
  float* a0 = gW + P;    // NP
  float* gy = a0 + NP;   // NP: output, then its gradient
  float* z1 = gy + NP;   // C*NP: pre-activation, then gradient
  float* a1 = z1 + C * NP;
  float* z2 = a1 + C * NP;
  float* a2 = z2 + C * NP;
  __shared__ float red[32];
  load_weights(W, sW, C);
  for (int p = threadIdx.x; p < P; p += blockDim.x) gW[p] = 0.f;
  const int n = threadIdx.x;
  const bool act = n < NP;
  const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
  const unsigned msk = act ? tap_mask<NQ>(i, j, k) : 0u;
  float lsum = 0.f;
  __syncthreads();
  for (int64_t e = blockIdx.x; e < E; e += gridDim.x) {
    if (act) a0[n] = in[e * NP + n];
    __syncthreads();
    if (act) {
      float acc[C];
      conv_fwd<NQ, 1, C>(a0, sW, n, msk, acc);
#pragma unroll
      for (int co = 0; co < C; ++co) {
        z1[co * NP + n] = acc[co];
        a1[co * NP + n] = gelu(acc[co]);
      }
    }
    __syncthreads();
    if (act) {
      float acc[C];
      conv_fwd<NQ, C, C>(a1, sW + o2, n, msk, acc);
#pragma unroll
      for (int co = 0; co < C; ++co) {
        z2[co * NP + n] = acc[co];
        a2[co * NP + n] = gelu(acc[co]);
      }
    }
    __syncthreads();
    if (act) {
      float acc[1];
      conv_fwd<NQ, C, 1>(a2, sW + o3, n, msk, acc);
      const float d = acc[0] - target[e * NP + n];
      lsum += d * d;
      gy[n] = gscale * d;  // d loss / d y
    }
    __syncthreads();
    // layer 3 weights, then gradient into z2 (in place)
    accum_wgrad<NQ>(gy, a2, gW + o3, C, 1);
    if (act) {
      float acc[C];
      conv_bwd_data<NQ, C, 1>(gy, sW + o3, n, msk, acc);
#pragma unroll
      for (int ci = 0; ci < C; ++ci) z2[ci * NP + n] = acc[ci] * gelu_grad(z2[ci * NP + n]);
    }
    __syncthreads();
    accum_wgrad<NQ>(z2, a1, gW + o2, C, C);
    if (act) {
      float acc[C];
      conv_bwd_data<NQ, C, C>(z2, sW + o2, n, msk, acc);
#pragma unroll
      for (int ci = 0; ci < C; ++ci) z1[ci * NP + n] = acc[ci] * gelu_grad(z1[ci * NP + n]);
    }
    __syncthreads();
    accum_wgrad<NQ>(z1, a0, gW, 1, C);
    __syncthreads();
  }
  for (int p = threadIdx.x; p < P; p += blockDim.x) gpart[(int64_t)blockIdx.x * P + p] = gW[p];
  const float ls = block_sum_f(lsum, red);
  if (threadIdx.x == 0) lpart[blockIdx.x] = ls;
}

// grad[p] = sum_b gpart[b][p] in block order; loss likewise
__global__ void k_net_reduce(int P, int nb, const float* __restrict__ gpart,
                             const float* __restrict__ lpart, float* __restrict__ grad,
                             float* __restrict__ loss, float lscale)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < P) {
    float s = 0.f;
    for (int b = 0; b < nb; ++b) s += gpart[(int64_t)b * P + p];
    grad[p] = s;
  }
  if (p == 0) {
    float s = 0.f;
    for (int b = 0; b < nb; ++b) s += lpart[b];
    *loss = s * lscale;
  }
}

__global__ void k_adam(int P, float* __restrict__ W, __nv_bfloat16* __restrict__ Wbf,
                       float* __restrict__ m, float* __restrict__ v, const float* __restrict__ g,
                       float lr, float b1, float b2, float eps, float c1, float c2)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const float gp = g[p];
  const float mp = b1 * m[p] + (1.f - b1) * gp;
  const float vp = b2 * v[p] + (1.f - b2) * gp * gp;
  m[p] = mp;
  v[p] = vp;
  const float w = W[p] - lr * (mp / c1) / (sqrtf(vp / c2) + eps);
  W[p] = w;
  Wbf[p] = __float2bfloat16_rn(w);
}

__global__ void k_to_bf16(int P, const float* W, __nv_bfloat16* Wbf)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < P) Wbf[p] = __float2bfloat16_rn(W[p]);
}

// in = h r_e / s_e ; target = (e_e - invDiag r_e) / (h s_e), h = sqrt(invDiag) per node
// (1 without invDiag), s_e = RMS of h r over element e
__global__ void k_prepare_pairs(int Np, int64_t Efield, const float* __restrict__ r,
                                const float* __restrict__ err, const float* __restrict__ invDiag,
                                float* __restrict__ in, float* __restrict__ target)
{
  __shared__ float red[32];
  const int64_t e = blockIdx.x;
  float ss = 0.f;
  for (int n = threadIdx.x; n < Np; n += blockDim.x) {
    const float h = invDiag ? sqrtf(invDiag[(e % Efield) * Np + n]) : 1.f;
    const float v = h * r[e * Np + n];
    ss += v * v;
  }
  const float s = sqrtf(block_sum_f(ss, red) / Np);
  const float inv = s > 0.f ? 1.f / s : 0.f;
  for (int n = threadIdx.x; n < Np; n += blockDim.x) {
    const int64_t id = e * Np + n;
    const float d = invDiag ? invDiag[(e % Efield) * Np + n] : 1.f;
    const float h = invDiag ? sqrtf(d) : 1.f;
    const float rv = r[id];
    const float dj = invDiag ? d * rv : 0.f;
    in[id] = h * rv * inv;
    target[id] = (h > 0.f && s > 0.f) ? (err[id] - dj) / (h * s) : 0.f;
  }
}

// Element-local correction of a residual: on each element's interior nodes
// (not shared with any other element) the solution y of the element Helmholtz
// problem A_II y = r_I with y = 0 on the element boundary (CG in FP32, one CTA
// per element, thread (i,j) owns the k-column); on the element-boundary nodes
// the Jacobi value invDiag * r.  This block solve is the linear map a local
// network can represent; PCG with it takes ~1.6x fewer iterations than Jacobi.
template <int NQ>
__host__ __device__ constexpr int lc_threads() { return (NQ * NQ + 31) / 32 * 32; }

template <int NQ>
__global__ void __launch_bounds__(lc_threads<NQ>())
k_local_correction(int64_t Esel, int64_t E, const int32_t* __restrict__ elems, const double* __restrict__ ggeo,
                   const float* __restrict__ Dg, const double* __restrict__ lambda, int64_t offset,
                   const float* __restrict__ r, const float* __restrict__ invDiag,
                   float* __restrict__ y, int iters, float tol)
{
  constexpr int NQ2 = NQ * NQ, NP = NQ2 * NQ, NW = lc_threads<NQ>() / 32;
  __shared__ float sD[NQ][NQ], sp[NP], sGr[NP], sGs[NP];
  __shared__ float red[NW];
  const int tid = threadIdx.x;
  const bool act = tid < NQ2;                 // lanes past the face only join the sums
  const int ij = act ? tid : 0, i = ij % NQ, j = ij / NQ;
  for (int t = tid; t < NQ2; t += blockDim.x) sD[t / NQ][t % NQ] = Dg[t];
  const bool ij_int = act && i > 0 && i < NQ - 1 && j > 0 && j < NQ - 1;
  auto bsum = [&](float v) {  // block sum in a fixed order
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    float s = 0.f;
#pragma unroll
    for (int w = 0; w < NW; ++w) s += red[w];
    return s;
  };
  for (int64_t b = blockIdx.x; b < Esel; b += gridDim.x) {
    const int64_t e = elems[b];
    if (e < 0 || e >= E) {  // not an element of this mesh: the row is left as zeros
      if (act)
        for (int k = 0; k < NQ; ++k) y[b * NP + k * NQ2 + ij] = 0.f;
      continue;
    }
    const double* g = ggeo + e * 7 * NP + ij;
    float G[7][NQ], l0[NQ], l1[NQ], rr_[NQ], x[NQ], res[NQ], p[NQ], Ap[NQ];
    bool in_k[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
#pragma unroll
      for (int sl = 0; sl < 7; ++sl) G[sl][k] = (float)g[sl * NP + k * NQ2];
      l0[k] = (float)lambda[e * NP + k * NQ2 + ij];
      l1[k] = (float)lambda[e * NP + k * NQ2 + ij + offset];
      in_k[k] = ij_int && k > 0 && k < NQ - 1;
      rr_[k] = r[b * NP + k * NQ2 + ij];
      x[k] = 0.f;
      res[k] = in_k[k] ? rr_[k] : 0.f;
      p[k] = res[k];
    }
    float rho = 0.f;
#pragma unroll
    for (int k = 0; k < NQ; ++k) rho += res[k] * res[k];
    rho = bsum(rho);
    const float rho0 = rho;
    for (int it = 0; it < iters && rho > tol * tol * rho0 && rho > 0.f; ++it) {
      // Ap = A p on the element, restricted to its interior nodes
      if (act) {
#pragma unroll
        for (int k = 0; k < NQ; ++k) sp[k * NQ2 + ij] = p[k];
      }
      __syncthreads();
      float gt[NQ];
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        float qr = 0.f, qs = 0.f, qt = 0.f;
#pragma unroll
        for (int m = 0; m < NQ; ++m) {
          qr += sD[i][m] * sp[k * NQ2 + j * NQ + m];
          qs += sD[j][m] * sp[k * NQ2 + m * NQ + i];
          qt += sD[k][m] * p[m];
        }
        if (act) {
          sGr[k * NQ2 + ij] = l0[k] * (G[1][k] * qr + G[2][k] * qs + G[3][k] * qt);
          sGs[k * NQ2 + ij] = l0[k] * (G[2][k] * qr + G[4][k] * qs + G[5][k] * qt);
        }
        gt[k] = l0[k] * (G[3][k] * qr + G[5][k] * qs + G[6][k] * qt);
      }
      __syncthreads();
      float pAp = 0.f;
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        float ak = G[0][k] * l1[k] * p[k];
#pragma unroll
        for (int m = 0; m < NQ; ++m)
          ak += sD[m][i] * sGr[k * NQ2 + j * NQ + m] + sD[m][j] * sGs[k * NQ2 + m * NQ + i] +
                sD[m][k] * gt[m];
        Ap[k] = in_k[k] ? ak : 0.f;
        pAp += p[k] * Ap[k];
      }
      pAp = bsum(pAp);
      const float alpha = pAp > 0.f ? rho / pAp : 0.f;
      float rho1 = 0.f;
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        x[k] += alpha * p[k];
        res[k] -= alpha * Ap[k];
        rho1 += res[k] * res[k];
      }
      rho1 = bsum(rho1);
      const float beta = rho1 / rho;
      rho = pAp > 0.f ? rho1 : 0.f;
#pragma unroll
      for (int k = 0; k < NQ; ++k) p[k] = res[k] + beta * p[k];
    }
    if (act) {
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const int64_t id = b * NP + k * NQ2 + ij;
        y[id] = in_k[k] ? x[k] : invDiag[id] * rr_[k];
      }
    }
    __syncthreads();
  }
}

template <int NQ, int C>
constexpr int infer_smem() { return (nparams(C) + np_of(NQ) * (1 + 2 * C)) * 4; }
template <int NQ, int C>
constexpr int train_smem() { return (2 * nparams(C) + np_of(NQ) * (2 + 4 * C)) * 4; }

template <int NQ, int C>
int run_infer(const nekb_net* net, int64_t Etot, int64_t Efield, const float* r, const float* w,
              const float* invDiag, float* out, int normalize, const int* skip, cudaStream_t s)
{
  constexpr int SM = infer_smem<NQ, C>();
  static SmemOptIn smem_opt;
  NEKB_TRY(smem_opt.ensure(k_net_infer<NQ, C>, SM));
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int per_sm = 0;
  NEKB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_net_infer<NQ, C>, threads_of(NQ), SM));
  int64_t grid = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
  if (grid > Etot) grid = Etot;
  if (grid < 1) return NEKB_OK;
  k_net_infer<NQ, C><<<(unsigned)grid, threads_of(NQ), SM, s>>>(
      Etot, Efield, net->Wbf.as<__nv_bfloat16>(), r, w, invDiag, out, normalize, skip);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

template <int NQ, int C>
int run_train(nekb_net* net, int64_t E, const float* in, const float* target, cudaStream_t s)
{
  constexpr int SM = train_smem<NQ, C>();
  static SmemOptIn smem_opt;
  NEKB_TRY(smem_opt.ensure(k_net_train<NQ, C>, SM));
  int64_t grid = net->gblocks;
  if (grid > E) grid = E;
  const float gscale = 2.0f / (float)(E * np_of(NQ));
  k_net_train<NQ, C><<<(unsigned)grid, threads_of(NQ), SM, s>>>(
      E, net->W.as<float>(), in, target, gscale, net->gpart.as<float>(), net->lpart.as<float>());
  NEKB_CUDA(cudaGetLastError());
  k_net_reduce<<<(net->P + 255) / 256, 256, 0, s>>>(net->P, (int)grid, net->gpart.as<float>(),
                                                    net->lpart.as<float>(), net->grad.as<float>(),
                                                    net->loss.as<float>(),
                                                    1.0f / (float)(E * np_of(NQ)));
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

#define NEKB_NET_DISPATCH(FN, ...)                                          \
  switch (net->Nq * 100 + net->C) {                                         \
    case 416: return FN<4, 16>(__VA_ARGS__);                                \
    case 408: return FN<4, 8>(__VA_ARGS__);                                 \
    case 616: return FN<6, 16>(__VA_ARGS__);                                \
    case 816: return FN<8, 16>(__VA_ARGS__);                                \
    case 808: return FN<8, 8>(__VA_ARGS__);                                 \
    case 804: return FN<8, 4>(__VA_ARGS__);                                 \
  }                                                                         \
  return fail(NEKB_ERR_UNSUPPORTED, "net: Nq=%d C=%d not built (Nq 4/6/8, C 4/8/16)", net->Nq, net->C);

// the tensor-core kernel NEKB_NET_TENSOR selects
constexpr int kTensorDefault = NEKB_NET_TENSOR_TC5;

int net_infer(const nekb_net* net, int64_t Etot, int64_t Efield, const float* r, const float* w,
              const float* invDiag, float* out, int normalize, const int* skip, cudaStream_t s)
{
  const int mode = net->inference == NEKB_NET_TENSOR ? kTensorDefault : net->inference;
  if (mode == NEKB_NET_TENSOR_TC5 && net_tc_supported(net->Nq, net->C))
    return net_infer_tc5(net->Wbf.as<__nv_bfloat16>(), Etot, Efield, r, w, invDiag, out, normalize,
                         skip, s);
  if (mode == NEKB_NET_TENSOR_SYNC && net_tc_supported(net->Nq, net->C))
    return net_infer_tc(net->Wbf.as<__nv_bfloat16>(), Etot, Efield, r, w, invDiag, out, normalize,
                        skip, s);
  NEKB_NET_DISPATCH(run_infer, net, Etot, Efield, r, w, invDiag, out, normalize, skip, s)
}

// the kernel net_infer launches: 0 FP32 cores, else the tensor-core mode
int resolved_mode(const nekb_net* net)
{
  const int mode = net->inference == NEKB_NET_TENSOR ? kTensorDefault : net->inference;
  if ((mode == NEKB_NET_TENSOR_TC5 || mode == NEKB_NET_TENSOR_SYNC) && net_tc_supported(net->Nq, net->C))
    return mode;
  return NEKB_NET_FP32;
}

int net_train(nekb_net* net, int64_t E, const float* in, const float* target, cudaStream_t s)
{
  NEKB_NET_DISPATCH(run_train, net, E, in, target, s)
}

bool net_supported(int Nq, int C)
{
  const int key = Nq * 100 + C;
  return key == 416 || key == 408 || key == 616 || key == 816 || key == 808 || key == 804;
}

}  // namespace

bool net_takes_update(const nekb_net* net) { return net && resolved_mode(net) == NEKB_NET_TENSOR_TC5; }

int net_precondition_update(nekb_bp* bp, nekb_net* net, const NetUpdate& up, float* r, float* z,
                            const float* invDiag, const float* w, const int* skip, cudaStream_t s)
{
  if (!net_takes_update(net)) return fail(NEKB_ERR_UNSUPPORTED, "net: the folded update needs the tcgen05 kernel");
  if (net->Nq != bp->Nq) return fail(NEKB_ERR_INVALID, "net order Nq=%d differs from the mesh's %d", net->Nq, bp->Nq);
  NEKB_TRY(net_infer_tc5(net->Wbf.as<__nv_bfloat16>(), bp->Nfields * bp->E, bp->E, r, w, invDiag, z,
                         kNetNormalize | kNetAddJacobi, skip, s, &up));
  NEKB_TRY(launch_gs_add(bp->ogs, bp->Nfields, bp->offset, z, NEKB_FLOAT, skip, s));
  NEKB_TRY(launch_mask(bp->Nmasked, bp->mask.as<int32_t>(), bp->Nfields, bp->offset, z, NEKB_FLOAT,
                       skip, s));
  return NEKB_OK;
}

NetSignature net_signature(const nekb_net* net)
{
  if (!net) return NetSignature{nullptr, nullptr, 0};
  return NetSignature{net, net->Wbf.p, (net->Nq * 100 + net->C) * 8 + resolved_mode(net)};
}

int net_precondition(nekb_bp* bp, nekb_net* net, const float* r, float* z, const float* invDiag,
                     const float* w, const int* skip, cudaStream_t s)
{
  if (!net) return fail(NEKB_ERR_INVALID, "learned preconditioner: no network");
  if (net->Nq != bp->Nq) return fail(NEKB_ERR_INVALID, "net order Nq=%d differs from the mesh's %d", net->Nq, bp->Nq);
  // z = w (h s net + invDiag r) per element copy, then assembled and masked
  NEKB_TRY(net_infer(net, bp->Nfields * bp->E, bp->E, r, w, invDiag, z,
                     kNetNormalize | kNetAddJacobi, skip, s));
  NEKB_TRY(launch_gs_add(bp->ogs, bp->Nfields, bp->offset, z, NEKB_FLOAT, skip, s));
  NEKB_TRY(launch_mask(bp->Nmasked, bp->mask.as<int32_t>(), bp->Nfields, bp->offset, z, NEKB_FLOAT,
                       skip, s));
  return NEKB_OK;
}

}  // namespace nekb

using namespace nekb;

static int net_alloc(nekb_net* net, int Nq, int C)
{
  net->Nq = Nq;
  net->Np = Nq * Nq * Nq;
  net->C = C;
  net->P = nparams(C);
  int dev = 0, sms = 152;
  NEKB_CUDA(cudaGetDevice(&dev));
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  net->gblocks = sms;
  NEKB_TRY(net->W.ensure(sizeof(float) * net->P));
  NEKB_TRY(net->Wbf.ensure(sizeof(__nv_bfloat16) * net->P));
  NEKB_TRY(net->m.ensure(sizeof(float) * net->P));
  NEKB_TRY(net->v.ensure(sizeof(float) * net->P));
  NEKB_TRY(net->grad.ensure(sizeof(float) * net->P));
  NEKB_TRY(net->gpart.ensure(sizeof(float) * net->P * (size_t)net->gblocks));
  NEKB_TRY(net->lpart.ensure(sizeof(float) * net->gblocks));
  NEKB_TRY(net->loss.ensure(sizeof(float)));
  NEKB_CUDA(cudaMemset(net->m.p, 0, sizeof(float) * net->P));
  NEKB_CUDA(cudaMemset(net->v.p, 0, sizeof(float) * net->P));
  return NEKB_OK;
}

static int net_upload(nekb_net* net, const float* w)
{
  NEKB_CUDA(cudaMemcpy(net->W.p, w, sizeof(float) * net->P, cudaMemcpyHostToDevice));
  k_to_bf16<<<(net->P + 255) / 256, 256>>>(net->P, net->W.as<float>(), net->Wbf.as<__nv_bfloat16>());
  NEKB_CUDA(cudaGetLastError());
  NEKB_CUDA(cudaDeviceSynchronize());
  return NEKB_OK;
}

template <int NQ>
static void launch_local_correction(int64_t n, const int32_t* elems, const nekb_bp* bp,
                                    const double* lambda, const float* r, const float* invDiag,
                                    float* y, int iters, float tol, cudaStream_t s)
{
  const unsigned g = (unsigned)std::min<int64_t>(n, 152 * 32);
  k_local_correction<NQ><<<g, lc_threads<NQ>(), 0, s>>>(
      n, bp->E, elems, bp->ggeo.as<double>(), bp->Df.as<float>(), lambda, bp->offset, r, invDiag, y,
      iters, tol);
}

extern "C" {

nekb_net* nekb_net_create(int Nq, int channels, int layers, uint64_t seed, int* status)
{
  int st = NEKB_OK;
  nekb_net* net = nullptr;
  if (layers != 3) {
    st = fail(NEKB_ERR_UNSUPPORTED, "net: %d layers (3 are built)", layers);
  } else if (!net_supported(Nq, channels)) {
    st = fail(NEKB_ERR_UNSUPPORTED, "net: Nq=%d C=%d not built (Nq 4/6/8, C 4/8/16)", Nq, channels);
  } else {
    net = new nekb_net();
    st = net_alloc(net, Nq, channels);
    if (st == NEKB_OK) {
      // uniform init U[-b, b], b = sqrt(6 / fan_in); the last layer scaled by 0.1
      // so the untrained network starts close to the plain Jacobi preconditioner
      std::vector<float> w(net->P);
      const int C = channels, o2 = kTaps * C, o3 = kTaps * C + kTaps * C * C;
      for (int p = 0; p < net->P; ++p) {
        const double fan_in = p < o2 ? kTaps : (double)kTaps * C;
        double b = std::sqrt(6.0 / fan_in);
        if (p >= o3) b *= 0.1;
        w[p] = (float)((2.0 * uniform01(seed, 77, (uint64_t)p) - 1.0) * b);
      }
      st = net_upload(net, w.data());
    }
    if (st != NEKB_OK) {
      delete net;
      net = nullptr;
    }
  }
  if (status) *status = st;
  return net;
}

void nekb_net_free(nekb_net* net) { delete net; }

int nekb_net_set_inference(nekb_net* net, int mode)
{
  if (!net || mode < NEKB_NET_FP32 || mode > NEKB_NET_TENSOR_TC5)
    return fail(NEKB_ERR_INVALID, "net inference: bad handle or mode %d", mode);
  net->inference = mode;
  return NEKB_OK;
}

int nekb_net_inference(const nekb_net* net)
{
  if (!net) return fail(NEKB_ERR_INVALID, "net inference: NULL handle");
  if (net->inference != NEKB_NET_FP32 && net_tc_supported(net->Nq, net->C)) return net->inference;
  return NEKB_NET_FP32;
}

int nekb_net_num_params(const nekb_net* net) { return net ? net->P : 0; }

int nekb_net_get_weights(const nekb_net* net, float* w)
{
  if (!net || !w) return fail(NEKB_ERR_INVALID, "net: NULL");
  NEKB_CUDA(cudaMemcpy(w, net->W.p, sizeof(float) * net->P, cudaMemcpyDeviceToHost));
  return NEKB_OK;
}

int nekb_net_set_weights(nekb_net* net, const float* w)
{
  if (!net || !w) return fail(NEKB_ERR_INVALID, "net: NULL");
  return net_upload(net, w);
}

int nekb_net_raise_copy_timeout(void) { return net_tc_raise_copy_timeout(); }

int nekb_net_forward(nekb_net* net, int64_t E, const float* in, float* out, void* stream)
{
  if (!net || (E > 0 && (!in || !out)) || E < 0) return fail(NEKB_ERR_INVALID, "net forward: bad arguments");
  if (E == 0) return NEKB_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  NEKB_TRY(net_infer(net, E, E, in, nullptr, nullptr, out, 0, nullptr, s));
  if (nekb_net_inference(net) != NEKB_NET_FP32) {
    NEKB_CUDA(cudaStreamSynchronize(s));
    return net_tc_copy_timeout();
  }
  return NEKB_OK;
}

int nekb_net_gradient(nekb_net* net, int64_t E, const float* in, const float* target, float* grad,
                      float* loss, void* stream)
{
  if (!net || E <= 0 || !in || !target) return fail(NEKB_ERR_INVALID, "net gradient: bad arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  NEKB_TRY(net_train(net, E, in, target, s));
  if (grad) NEKB_CUDA(cudaMemcpyAsync(grad, net->grad.p, sizeof(float) * net->P, cudaMemcpyDeviceToHost, s));
  if (loss) NEKB_CUDA(cudaMemcpyAsync(loss, net->loss.p, sizeof(float), cudaMemcpyDeviceToHost, s));
  NEKB_CUDA(cudaStreamSynchronize(s));
  return NEKB_OK;
}

int nekb_net_train_step(nekb_net* net, int64_t E, const float* in, const float* target, float lr,
                        float* loss, void* stream)
{
  if (!net || E <= 0 || !in || !target || !(lr > 0)) return fail(NEKB_ERR_INVALID, "net train: bad arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  NEKB_TRY(net_train(net, E, in, target, s));
  net->step++;
  const float c1 = 1.f - std::pow(net->beta1, (float)net->step);
  const float c2 = 1.f - std::pow(net->beta2, (float)net->step);
  k_adam<<<(net->P + 255) / 256, 256, 0, s>>>(net->P, net->W.as<float>(), net->Wbf.as<__nv_bfloat16>(),
                                               net->m.as<float>(), net->v.as<float>(),
                                               net->grad.as<float>(), lr, net->beta1, net->beta2,
                                               net->eps, c1, c2);
  NEKB_CUDA(cudaGetLastError());
  if (loss) {
    NEKB_CUDA(cudaMemcpyAsync(loss, net->loss.p, sizeof(float), cudaMemcpyDeviceToHost, s));
    NEKB_CUDA(cudaStreamSynchronize(s));
  }
  return NEKB_OK;
}

int nekb_net_prepare_pairs(int Np, int64_t E, int64_t Efield, const float* r, const float* err,
                           const float* invDiag, float* in, float* target, void* stream)
{
  if (Np <= 0 || E < 0 || Efield <= 0 || (E > 0 && (!r || !err || !in || !target)))
    return fail(NEKB_ERR_INVALID, "prepare pairs: bad arguments");
  if (E == 0) return NEKB_OK;
  if (E > 0x7fffffff) return fail(NEKB_ERR_INVALID, "prepare pairs: too many elements");
  k_prepare_pairs<<<(unsigned)E, 256, 0, static_cast<cudaStream_t>(stream)>>>(Np, Efield, r, err, invDiag, in, target);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int nekb_bp_local_correction(nekb_bp* bp, const double* lambda, const int32_t* elems, int64_t n,
                             const float* r, const float* invDiag, float* y, int iters, float tol)
{
  if (!bp || n < 0 || iters < 0 || !(tol >= 0.f) ||
      (n > 0 && (!lambda || !elems || !r || !invDiag || !y)))
    return fail(NEKB_ERR_INVALID, "local correction: bad arguments");
  if (n == 0) return NEKB_OK;
  cudaStream_t s = bp->stream;
  switch (bp->Nq) {
    case 3: launch_local_correction<3>(n, elems, bp, lambda, r, invDiag, y, iters, tol, s); break;
    case 4: launch_local_correction<4>(n, elems, bp, lambda, r, invDiag, y, iters, tol, s); break;
    case 5: launch_local_correction<5>(n, elems, bp, lambda, r, invDiag, y, iters, tol, s); break;
    case 6: launch_local_correction<6>(n, elems, bp, lambda, r, invDiag, y, iters, tol, s); break;
    case 7: launch_local_correction<7>(n, elems, bp, lambda, r, invDiag, y, iters, tol, s); break;
    case 8: launch_local_correction<8>(n, elems, bp, lambda, r, invDiag, y, iters, tol, s); break;
    default:
      return fail(NEKB_ERR_UNSUPPORTED, "local correction: Nq=%d not built (3..8)", bp->Nq);
  }
  NEKB_CUDA(cudaGetLastError());
  NEKB_CUDA(cudaStreamSynchronize(s));
  return NEKB_OK;
}

// versioned checkpoint: magic, version, Nq, C, layers, P, step, weights, Adam m, v, CRC32
static uint32_t crc32(const unsigned char* p, size_t n, uint32_t c = 0xffffffffu)
{
  for (size_t i = 0; i < n; ++i) {
    c ^= p[i];
    for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
  }
  return c;
}

int nekb_net_save(const nekb_net* net, const char* path)
{
  if (!net || !path) return fail(NEKB_ERR_INVALID, "net save: NULL");
  const int P = net->P;
  std::vector<float> buf(3 * (size_t)P);
  NEKB_CUDA(cudaMemcpy(buf.data(), net->W.p, sizeof(float) * P, cudaMemcpyDeviceToHost));
  NEKB_CUDA(cudaMemcpy(buf.data() + P, net->m.p, sizeof(float) * P, cudaMemcpyDeviceToHost));
  NEKB_CUDA(cudaMemcpy(buf.data() + 2 * P, net->v.p, sizeof(float) * P, cudaMemcpyDeviceToHost));
  int32_t hdr[6] = {0x4e454b4e /* "NKEN" */, 1, net->Nq, net->C, 3, P};
  int64_t step = net->step;
  uint32_t c = crc32((const unsigned char*)hdr, sizeof(hdr));
  c = crc32((const unsigned char*)&step, sizeof(step), c);
  c = crc32((const unsigned char*)buf.data(), sizeof(float) * buf.size(), c);
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(NEKB_ERR_INVALID, "net save: cannot open %s", path);
  bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1 && std::fwrite(&step, sizeof(step), 1, f) == 1 &&
            std::fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size() &&
            std::fwrite(&c, sizeof(c), 1, f) == 1;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? NEKB_OK : fail(NEKB_ERR_INVALID, "net save: write failed for %s", path);
}

nekb_net* nekb_net_load(const char* path, int* status)
{
  int st = NEKB_OK;
  nekb_net* net = nullptr;
  FILE* f = path ? std::fopen(path, "rb") : nullptr;
  int32_t hdr[6] = {0};
  int64_t step = 0;
  std::vector<float> buf;
  uint32_t c_file = 0;
  if (!f) {
    st = fail(NEKB_ERR_INVALID, "net load: cannot open %s", path ? path : "(null)");
  } else if (std::fread(hdr, sizeof(hdr), 1, f) != 1 || hdr[0] != 0x4e454b4e || hdr[1] != 1 ||
             hdr[4] != 3 || !net_supported(hdr[2], hdr[3]) || hdr[5] != nparams(hdr[3])) {
    st = fail(NEKB_ERR_INVALID, "net load: %s is not a version-1 network checkpoint", path);
  } else {
    buf.resize(3 * (size_t)hdr[5]);
    if (std::fread(&step, sizeof(step), 1, f) != 1 ||
        std::fread(buf.data(), sizeof(float), buf.size(), f) != buf.size() ||
        std::fread(&c_file, sizeof(c_file), 1, f) != 1) {
      st = fail(NEKB_ERR_INVALID, "net load: %s is truncated", path);
    } else {
      uint32_t c = crc32((const unsigned char*)hdr, sizeof(hdr));
      c = crc32((const unsigned char*)&step, sizeof(step), c);
      c = crc32((const unsigned char*)buf.data(), sizeof(float) * buf.size(), c);
      if (c != c_file) st = fail(NEKB_ERR_INVALID, "net load: checksum mismatch in %s", path);
    }
  }
  if (f) std::fclose(f);
  if (st == NEKB_OK) {
    net = new nekb_net();
    st = net_alloc(net, hdr[2], hdr[3]);
    if (st == NEKB_OK) st = net_upload(net, buf.data());
    if (st == NEKB_OK) {
      const int P = net->P;
      net->step = step;
      if (cudaMemcpy(net->m.p, buf.data() + P, sizeof(float) * P, cudaMemcpyHostToDevice) != cudaSuccess ||
          cudaMemcpy(net->v.p, buf.data() + 2 * P, sizeof(float) * P, cudaMemcpyHostToDevice) != cudaSuccess)
        st = fail(NEKB_ERR_CUDA, "net load: upload failed");
    }
    if (st != NEKB_OK) {
      delete net;
      net = nullptr;
    }
  }
  if (status) *status = st;
  return net;
}

}  // extern "C"
