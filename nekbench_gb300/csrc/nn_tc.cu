// Warp-level tensor-core inference of the learned element preconditioner for
// N=7 (Nq=8, 512 nodes) and 16 channels (NEKB_NET_TENSOR_SYNC; nn_tc5.cu holds
// the tcgen05 kernel): the three 3x3x3 convolutions of an element as implicit
// GEMMs on the BF16 tensor cores (mma.m16n8k16, FP32 accumulation).
//
// One CTA of 4 warps per element at a time (persistent grid).  Node n =
// i + 8j + 64k; warp w owns the 16 nodes j in {2w, 2w+1}, i = 0..7 of every
// plane k (one m16 row tile per plane).
//   layer 1 (1 -> 16):  A[node][tap] gathered from the scaled residual (27 taps
//                        padded to K=32), B = W1[tap][co].
//   layer 2 (16 -> 16): per tap a GEMM with K = 16 input channels.  The
//                        activation tile of plane p shifted by (di,dj) is loaded
//                        once (ldmatrix, out-of-element rows point to a zero
//                        row) and multiplied into the accumulators of output
//                        planes p+1, p, p-1 (taps dk = -1, 0, +1); the 27 weight
//                        fragments stay in registers for the whole kernel.
//   layer 3 (16 -> 1):  U[node][tap] = act[node][:] . W3[:][tap] (N = 27 taps
//                        padded to 32), then out[n] = sum_t U[n + off_t][t].
// Activations are rounded to BF16 between layers (GELU outputs and the scaled
// input); weights are BF16; all sums are FP32.  GELU uses the tanh form with
// the hardware tanh approximation.
// No counterpart in the reference.
#include "nn.h"

#include <cuda_bf16.h>

namespace nekb {
namespace {

constexpr int kNq = 8, kNp = 512, kTaps = 27, kThreads = 128;
constexpr int kUStride = 516;  // floats; makes the fragment stores of U conflict-free
constexpr int kO2 = kTaps * 16, kO3 = kTaps * 16 + kTaps * 16 * 16;

// shared memory (bytes)
constexpr int kSmAct = 0;                                // [512 nodes][16 ch] bf16, swizzled
constexpr int kSmZero = kSmAct + kNp * 32;               // 32 zero bytes
constexpr int kSmA0 = kSmZero + 32;                      // scaled input, 512 floats
constexpr int kSmH = kSmA0 + kNp * 4;                    // sqrt(invDiag), 512 floats
constexpr int kSmU = kSmH + kNp * 4;                     // [27][kUStride] floats
constexpr int kSmRed = kSmU + kTaps * kUStride * 4;      // block-sum scratch
constexpr int kSmIn = kSmRed + 64;                       // [2 buffers][r, invDiag, w][512] floats
constexpr int kSmBar = kSmIn + 2 * 3 * kNp * 4;          // two mbarriers
constexpr int kSmTotal = kSmBar + 16;
constexpr int kRowBytes = kNp * 4;                       // one element row of a node array
constexpr long kWaitLimit = 1L << 22;                    // bounded mbarrier waits

// set when an input copy did not complete within kWaitLimit polls
__device__ int g_tc_copy_timeout;

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t (&r)[4])
{
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr)
               : "memory");
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
  asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi)
{
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ float gelu_tc(float x)
{
  const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  return 0.5f * x * (1.0f + t);
}

// byte offset of channel half `half` (channels 8*half .. 8*half+7) of node n;
// the halves of nodes with bit 2 set are swapped so that 8 consecutive nodes
// fall into 8 distinct 16-byte bank groups
__device__ __forceinline__ int act_off(int n, int half) { return n * 32 + ((half ^ ((n >> 2) & 1)) << 4); }

__device__ __forceinline__ uint32_t wpair(const uint16_t* W, int i0, int i1, bool v0, bool v1)
{
  const uint32_t lo = v0 ? W[i0] : 0u, hi = v1 ? W[i1] : 0u;
  return lo | (hi << 16);
}

// ---- bulk asynchronous copies of an element's input rows (cp.async.bulk with
// mbarrier completion): the next element's rows are fetched while the current
// one is computed
__device__ __forceinline__ void bar_init(uint32_t bar)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void bar_expect(uint32_t bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_row(uint32_t dst, const float* src, uint32_t bar)
{
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::
          "r"(dst), "l"(src), "r"((uint32_t)kRowBytes), "r"(bar)
      : "memory");
}

// true once the barrier has completed the phase with the given parity; false
// after kWaitLimit polls
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity)
{
  for (long it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ float block_sum4(float v, float* red)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  return red[0] + red[1] + red[2] + red[3];
}

__global__ void __launch_bounds__(kThreads, 2)
k_net_infer_tc(int64_t Etot, int64_t Efield, const __nv_bfloat16* __restrict__ Wbf,
               const float* __restrict__ r, const float* __restrict__ w,
               const float* __restrict__ invDiag, float* __restrict__ out, int normalize,
               const int* skip)
{
  if (skip != nullptr && *skip != 0) return;
  extern __shared__ __align__(128) unsigned char smem[];
  float* a0 = reinterpret_cast<float*>(smem + kSmA0);
  float* hs = reinterpret_cast<float*>(smem + kSmH);
  float* U = reinterpret_cast<float*>(smem + kSmU);
  float* red = reinterpret_cast<float*>(smem + kSmRed);
  const uint32_t act_s = smem_addr(smem + kSmAct), zero_s = smem_addr(smem + kSmZero);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, tig = lane & 3;
  const uint16_t* W = reinterpret_cast<const uint16_t*>(Wbf);
  if (tid < 8) reinterpret_cast<uint32_t*>(smem + kSmZero)[tid] = 0u;

  // weight fragments, loaded once.  B[k][n] of mma.m16n8k16: registers
  // {k = 2 tig, 2 tig + 1} and {k = 2 tig + 8, 2 tig + 9}, column n = g.
  uint32_t B1[2][2][2], B2[kTaps][2][2], B3[4][2];
#pragma unroll
  for (int ks = 0; ks < 2; ++ks)
#pragma unroll
    for (int nb = 0; nb < 2; ++nb)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int t = ks * 16 + 2 * tig + 8 * h, co = nb * 8 + g;
        B1[ks][nb][h] = wpair(W, co * kTaps + t, co * kTaps + t + 1, t < kTaps, t + 1 < kTaps);
      }
#pragma unroll
  for (int t = 0; t < kTaps; ++t)
#pragma unroll
    for (int nb = 0; nb < 2; ++nb)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int ci = 2 * tig + 8 * h, co = nb * 8 + g;
        B2[t][nb][h] = wpair(W, kO2 + (co * 16 + ci) * kTaps + t, kO2 + (co * 16 + ci + 1) * kTaps + t,
                             true, true);
      }
#pragma unroll
  for (int nb = 0; nb < 4; ++nb)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int ci = 2 * tig + 8 * h, t = nb * 8 + g;
      B3[nb][h] = wpair(W, kO3 + ci * kTaps + t, kO3 + (ci + 1) * kTaps + t, t < kTaps, t < kTaps);
    }

  // this lane's ldmatrix row: matrix m = lane/8 -> rows j = 2w + (m&1), i = lane%8,
  // channel half m>>1
  const int lm = lane >> 3, li = lane & 7, lj = 2 * warp + (lm & 1), lhalf = lm >> 1;
  // this thread's accumulator rows: i = g, j = 2w (c0,c1) and 2w+1 (c2,c3)
  const int jA = 2 * warp, jB = 2 * warp + 1;

  // input rows r, invDiag, w of an element: double-buffered in shared memory,
  // filled by bulk copies that complete on the buffer's mbarrier
  const float* inb = reinterpret_cast<const float*>(smem + kSmIn);
  const uint32_t in_s = smem_addr(smem + kSmIn), bar_s = smem_addr(smem + kSmBar);
  const uint32_t nrows = 1u + (invDiag ? 1u : 0u) + (w ? 1u : 0u);
  if (tid == 0) {
    bar_init(bar_s);
    bar_init(bar_s + 8);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  }
  __syncthreads();
  auto fetch = [&](int64_t el, int buf) {  // one thread issues the copies of element el
    const uint32_t bar = bar_s + 8 * buf, dst = in_s + buf * 3 * kRowBytes;
    bar_expect(bar, nrows * kRowBytes);
    bulk_row(dst, r + el * kNp, bar);
    if (invDiag) bulk_row(dst + kRowBytes, invDiag + (el % Efield) * kNp, bar);
    if (w) bulk_row(dst + 2 * kRowBytes, w + (el % Efield) * kNp, bar);
  };
  if (tid == 0 && (int64_t)blockIdx.x < Etot) fetch(blockIdx.x, 0);
  uint32_t parity0 = 0, parity1 = 0;
  int buf = 0;

  for (int64_t e = blockIdx.x; e < Etot; e += gridDim.x, buf ^= 1) {
    // the other buffer was released by the previous element's last barrier
    const bool next = e + gridDim.x < Etot;
    if (tid == 0 && next) {
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // reads of the buffer are done
      fetch(e + gridDim.x, buf ^ 1);
    }
    const bool ok = bar_wait(bar_s + 8 * buf, buf ? parity1 : parity0);
    if (buf) parity1 ^= 1u; else parity0 ^= 1u;
    if (__syncthreads_or(!ok)) {  // give up: wait (bounded) for the copy in flight, flag, return
      if (tid == 0) {
        if (next) bar_wait(bar_s + 8 * (buf ^ 1), buf ? parity0 : parity1);
        atomicExch(&g_tc_copy_timeout, 1);
      }
      return;
    }
    const float* rin = inb + buf * 3 * kNp;
    const float* din = rin + kNp;
    const float* win = rin + 2 * kNp;
    // ---- scaled input: a0 = h r / s
    float ss = 0.f;
#pragma unroll
    for (int c = 0; c < kNp / kThreads; ++c) {
      const int n = tid + c * kThreads;
      const float h = invDiag ? sqrtf(din[n]) : 1.f;
      const float v = h * rin[n];
      hs[n] = h;
      a0[n] = v;
      ss += v * v;
    }
    float s = 1.f;
    if (normalize & kNetNormalize) s = sqrtf(block_sum4(ss, red) / kNp);
    const float inv = s > 0.f ? 1.f / s : 0.f;
#pragma unroll
    for (int c = 0; c < kNp / kThreads; ++c) {
      const int n = tid + c * kThreads;
      a0[n] = __bfloat162float(__float2bfloat16_rn(a0[n] * inv));
    }
    __syncthreads();

    // ---- layer 1.  The thread's 8 taps t = 16 ks + 2 tig + {0, 1, 8, 9} are
    // fixed: their node offsets, k-shifts and in-plane validity for rows
    // (g, jA) and (g, jB) are set up once per element.
    int toff[8], tdk[8];
    unsigned okA = 0u, okB = 0u;
#pragma unroll
    for (int h = 0; h < 8; ++h) {
      const int t = (h >> 2) * 16 + 2 * tig + (h & 1) + ((h >> 1) & 1) * 8;
      const int di = t % 3 - 1, dj = (t / 3) % 3 - 1, dk = t / 9 - 1;
      toff[h] = di + kNq * dj + kNq * kNq * dk;
      tdk[h] = dk;
      const bool iok = t < kTaps && g + di >= 0 && g + di < kNq;
      if (iok && jA + dj >= 0 && jA + dj < kNq) okA |= 1u << h;
      if (iok && jB + dj >= 0 && jB + dj < kNq) okB |= 1u << h;
    }
#pragma unroll 1
    for (int k = 0; k < kNq; ++k) {
      const int nA0 = g + kNq * jA + kNq * kNq * k, nB0 = g + kNq * jB + kNq * kNq * k;
      float va[8], vb[8];
#pragma unroll
      for (int h = 0; h < 8; ++h) {
        const bool kok = (unsigned)(k + tdk[h]) < (unsigned)kNq;
        va[h] = (kok && ((okA >> h) & 1u)) ? a0[nA0 + toff[h]] : 0.f;
        vb[h] = (kok && ((okB >> h) & 1u)) ? a0[nB0 + toff[h]] : 0.f;
      }
      float acc[2][4] = {};
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
        uint32_t A[4];
        A[0] = pack2(va[4 * ks + 0], va[4 * ks + 1]);
        A[1] = pack2(vb[4 * ks + 0], vb[4 * ks + 1]);
        A[2] = pack2(va[4 * ks + 2], va[4 * ks + 3]);
        A[3] = pack2(vb[4 * ks + 2], vb[4 * ks + 3]);
#pragma unroll
        for (int nb = 0; nb < 2; ++nb) mma16816(acc[nb], A, B1[ks][nb][0], B1[ks][nb][1]);
      }
      const int nA = g + kNq * jA + kNq * kNq * k, nB = g + kNq * jB + kNq * kNq * k;
#pragma unroll
      for (int nb = 0; nb < 2; ++nb) {
        *reinterpret_cast<uint32_t*>(smem + kSmAct + act_off(nA, nb) + 4 * tig) =
            pack2(gelu_tc(acc[nb][0]), gelu_tc(acc[nb][1]));
        *reinterpret_cast<uint32_t*>(smem + kSmAct + act_off(nB, nb) + 4 * tig) =
            pack2(gelu_tc(acc[nb][2]), gelu_tc(acc[nb][3]));
      }
    }
    __syncthreads();

    // ---- layer 2: accumulators of all 8 planes in registers
    float acc[kNq][2][4];
#pragma unroll
    for (int q = 0; q < kNq; ++q)
#pragma unroll
      for (int nb = 0; nb < 2; ++nb)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[q][nb][c] = 0.f;
#pragma unroll
    for (int p = 0; p < kNq; ++p) {
#pragma unroll
      for (int dj = -1; dj <= 1; ++dj) {
#pragma unroll
        for (int di = -1; di <= 1; ++di) {
          const int i2 = li + di, j2 = lj + dj;
          const bool in = i2 >= 0 && i2 < kNq && j2 >= 0 && j2 < kNq;
          const uint32_t addr = in ? act_s + act_off(i2 + kNq * j2 + kNq * kNq * p, lhalf) : zero_s;
          uint32_t A[4];
          ldsm_x4(addr, A);
#pragma unroll
          for (int dk = -1; dk <= 1; ++dk) {
            const int q = p - dk;
            if (q < 0 || q >= kNq) continue;
            const int t = (di + 1) + 3 * (dj + 1) + 9 * (dk + 1);
            mma16816(acc[q][0], A, B2[t][0][0], B2[t][0][1]);
            mma16816(acc[q][1], A, B2[t][1][0], B2[t][1][1]);
          }
        }
      }
    }
    __syncthreads();  // every warp has finished reading the layer-1 activations
#pragma unroll
    for (int q = 0; q < kNq; ++q) {
      const int nA = g + kNq * jA + kNq * kNq * q, nB = g + kNq * jB + kNq * kNq * q;
#pragma unroll
      for (int nb = 0; nb < 2; ++nb) {
        *reinterpret_cast<uint32_t*>(smem + kSmAct + act_off(nA, nb) + 4 * tig) =
            pack2(gelu_tc(acc[q][nb][0]), gelu_tc(acc[q][nb][1]));
        *reinterpret_cast<uint32_t*>(smem + kSmAct + act_off(nB, nb) + 4 * tig) =
            pack2(gelu_tc(acc[q][nb][2]), gelu_tc(acc[q][nb][3]));
      }
    }
    __syncthreads();

    // ---- layer 3: U[t][n] = sum_ci act[n][ci] W3[ci][t]
#pragma unroll 1
    for (int k = 0; k < kNq; ++k) {
      uint32_t A[4];
      ldsm_x4(act_s + act_off(li + kNq * lj + kNq * kNq * k, lhalf), A);
      float u[4][4] = {};
#pragma unroll
      for (int nb = 0; nb < 4; ++nb) mma16816(u[nb], A, B3[nb][0], B3[nb][1]);
      const int nA = g + kNq * jA + kNq * kNq * k, nB = g + kNq * jB + kNq * kNq * k;
#pragma unroll
      for (int nb = 0; nb < 4; ++nb) {
        const int t = nb * 8 + 2 * tig;
        if (t < kTaps) {
          U[t * kUStride + nA] = u[nb][0];
          U[t * kUStride + nB] = u[nb][2];
        }
        if (t + 1 < kTaps) {
          U[(t + 1) * kUStride + nA] = u[nb][1];
          U[(t + 1) * kUStride + nB] = u[nb][3];
        }
      }
    }
    __syncthreads();

    // ---- out[n] = w (h s sum_t U[t][n + off_t] (+ invDiag r))
#pragma unroll
    for (int c = 0; c < kNp / kThreads; ++c) {
      const int n = tid + c * kThreads;
      const int i = n % kNq, j = (n / kNq) % kNq, k = n / (kNq * kNq);
      float o = 0.f;
#pragma unroll
      for (int t = 0; t < kTaps; ++t) {
        const int di = t % 3 - 1, dj = (t / 3) % 3 - 1, dk = t / 9 - 1;
        const int a = i + di, b = j + dj, cc = k + dk;
        if (a >= 0 && a < kNq && b >= 0 && b < kNq && cc >= 0 && cc < kNq)
          o += U[t * kUStride + n + di + kNq * dj + kNq * kNq * dk];
      }
      const float wn = w ? win[n] : 1.f;
      o *= hs[n] * s;
      if ((normalize & kNetAddJacobi) && invDiag) o += din[n] * rin[n];
      out[e * kNp + n] = wn * o;
    }
    __syncthreads();  // U, act, a0 and this input buffer are rewritten later
  }
}

}  // namespace

int net_tc_copy_timeout()
{
  int flag = 0, flag5 = 0;
  NEKB_CUDA(cudaMemcpyFromSymbol(&flag, g_tc_copy_timeout, sizeof(int)));
  if (flag) {
    const int zero = 0;
    NEKB_CUDA(cudaMemcpyToSymbol(g_tc_copy_timeout, &zero, sizeof(int)));
  }
  NEKB_TRY(net_tc5_take_timeout(&flag5));
  if (flag || flag5)
    return fail(NEKB_ERR_CUDA, "network: an input copy or a tensor-core operation did not complete in time");
  return NEKB_OK;
}

int net_tc_raise_copy_timeout()
{
  const int one = 1;
  NEKB_CUDA(cudaMemcpyToSymbol(g_tc_copy_timeout, &one, sizeof(int)));
  return net_tc5_raise_timeout();
}

bool net_tc_supported(int Nq, int C) { return Nq == kNq && C == 16; }

int net_infer_tc(const __nv_bfloat16* Wbf, int64_t Etot, int64_t Efield, const float* r,
                 const float* w, const float* invDiag, float* out, int normalize, const int* skip,
                 cudaStream_t s)
{
  // the bulk copies move whole element rows: 16-byte aligned arrays
  for (const void* p : {(const void*)r, (const void*)w, (const void*)invDiag})
    if (reinterpret_cast<uintptr_t>(p) % 16 != 0)
      return fail(NEKB_ERR_INVALID, "network: input arrays must be 16-byte aligned");
  static SmemOptIn smem_opt;
  NEKB_TRY(smem_opt.ensure(k_net_infer_tc, kSmTotal));
  int dev = 0, sms = 152, per_sm = 0;
  NEKB_CUDA(cudaGetDevice(&dev));
  NEKB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  NEKB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_net_infer_tc, kThreads, kSmTotal));
  // two CTAs fit an SM by the launch bounds and the shared-memory plan; the
  // occupancy query has reported one for such kernels
  static_assert(2 * (kSmTotal + 1024) <= 233472, "two CTAs fit one SM's shared memory");
  if (per_sm < 2) per_sm = 2;
  int64_t grid = (int64_t)sms * per_sm;
  if (grid > Etot) grid = Etot;
  if (grid < 1) return NEKB_OK;
  k_net_infer_tc<<<(unsigned)grid, kThreads, kSmTotal, s>>>(Etot, Efield, Wbf, r, w, invDiag, out,
                                                            normalize, skip);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

}  // namespace nekb
