// Learned element preconditioner for N=7 (Nq=8, 512 nodes), 16 channels, on
// the fifth-generation tensor cores: tcgen05.mma with operands in shared
// memory and accumulators in tensor memory (TMEM).
//
// Layout.  An element's nodes (i, j, k) are stored with one zero row of nodes
// before and after every j line-set and one zero plane before and after the
// k planes: padded row n' = i + 8 j' + 80 k', j' = j + 1 in 0..9, k' = k + 1
// in 0..9 (800 rows, plus 8 spare rows at both ends).  Activations are BF16,
// [row][16 channels], in the canonical no-swizzle K-major layout of core
// matrices (8 rows x 16 bytes): row group g = row/8, channel half h = c/8 at
// byte (2 g + h) * 128.  A shift of the input by (dj, dk) is then a shift of
// the A operand's start address by (8 dj + 80 dk) rows, i.e. whole row groups,
// and the padding supplies the zeros outside the element.
//
// Layer 2 (16 -> 16) as one GEMM per 128-row tile (5 tiles cover planes
// k = 0..7): K runs over (dj, dk, ci) -- nine MMAs of K = 16, one per shifted
// A -- and N over (di, co) = 48 columns:
//   V[n'][di][co] = sum_{dj,dk,ci} act[n' + 8 dj + 80 dk][ci] W[(di,dj,dk)][ci][co].
// The di shift is left to the epilogue: out(i) = sum_di V(i + di)[di], and
// node i +- 1 is lane +- 1 of the same warp (tile rows start at multiples of 8,
// so lane mod 8 = i), so two shuffles finish the convolution.  Layer 1
// (1 -> 16) uses an im2col of the 9 (di, dk) taps as its 16-wide K (three MMAs
// for dj = -1, 0, 1, N = 16) and layer 3 (16 -> 1) the layer-2 scheme with
// N = 16 (columns di = -1, 0, 1 used).  Every TMEM read-back stays in the
// reading warp's own 32 lanes: no shared-memory round trip of the partial sums.
//
// One CTA of 4 warps per element at a time, three CTAs per SM (persistent
// grid; 75 KB of shared memory and 128 TMEM columns each), so that each warp
// scheduler has three warps to switch between.  Thread 0 issues the MMAs of a
// layer tile by tile and commits each tile to its own mbarrier, so the
// epilogue of tile t (TMEM -> registers, shuffles, GELU, BF16, next layer's
// operand) overlaps the MMAs of the later tiles.  Layer 2's accumulators
// (5 tiles x 48 columns) cycle through two 48-column buffers: tile t + 2 is
// issued once every warp has read tile t.  The input staging is bordered with
// zeros in i and k, so the layer-1 im2col reads its nine taps without bounds
// tests; GELU's factor 1/2 rides in the next layer's weights (halved when
// staged).  Inputs are read straight from global memory.  Every wait is
// bounded; a wait that runs out sets a device flag, the CTA waits (bounded)
// for its operations in flight, frees its TMEM and returns.
//
// Arithmetic: BF16 weights and activations (the scaled input and both GELU
// outputs rounded to BF16), FP32 accumulation, the tanh form of GELU with the
// hardware tanh.  No counterpart in the reference.
#include "nn.h"

#include <cuda_bf16.h>

namespace nekb {
namespace {

constexpr int kNq = 8, kNp = 512, kTaps = 27, kThreads = 128;
constexpr int kO2 = kTaps * 16, kO3 = kTaps * 16 + kTaps * 16 * 16;
constexpr int kPlaneRows = 80;           // 8 i x 10 j' per padded plane
constexpr int kLead = 8;                 // spare rows before padded row 0
constexpr int kRows = 816;               // 8 + 800 + 8 storage rows
constexpr int kTiles = 5;                // 128-row tiles over padded rows 80..719
constexpr int kTile0 = kPlaneRows;       // first tile row (plane k' = 1)
constexpr int kActBytes = kRows * 32;    // one activation buffer
constexpr int kA0Rows = 10, kA0Plane = 80;  // bordered input: (i + 1) + 10 j + 80 (k + 1)

// shared memory (bytes)
constexpr int kSmW1 = 0;                         // 3 x [16 n][16 k] bf16
constexpr int kSmW2 = kSmW1 + 3 * 512;           // 9 x [48 n][16 k]
constexpr int kSmW3 = kSmW2 + 9 * 1536;          // 9 x [16 n][16 k]
constexpr int kSmX = kSmW3 + 9 * 512;            // layer-1 im2col, then layer-2 output (19968)
constexpr int kSmY = kSmX + kActBytes;           // layer-1 output
constexpr int kSmH = kSmY + kActBytes;           // sqrt(invDiag), 512 floats
constexpr int kSmA0 = kSmH + kNp * 4;            // scaled input, BF16, zero-bordered in i and k (800 x 2 bytes)
constexpr int kSmRed = kSmA0 + kNp * 4;          // block sums
constexpr int kSmBar = kSmRed + 64;              // 5 tile mbarriers
constexpr int kSmSlot = kSmBar + kTiles * 8;     // TMEM base address
constexpr int kSmTotal = kSmSlot + 16;
constexpr int kCtasPerSm = 3;
constexpr uint32_t kTmemCols = 128;              // layers 1 and 3: 5 x 16; layer 2: 2 x 48
constexpr long kWaitLimit = 1L << 22;

static_assert(kSmX % 256 == 0 && kSmY % 256 == 0, "operand buffers aligned");
static_assert(kCtasPerSm * (kSmTotal + 1024) <= 233472, "three CTAs fit one SM's shared memory");
static_assert(kCtasPerSm * kTmemCols <= 512, "the resident CTAs share the 512 TMEM columns");

// set when a wait (input copy or MMA) did not complete within kWaitLimit polls
__device__ int g_tc5_timeout;

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of (row, channel half) in an operand buffer
__device__ __forceinline__ int core_off(int row, int half) { return ((row >> 3) * 2 + half) * 128 + (row & 7) * 16; }

// shared-memory matrix descriptor: no swizzle, K-major; leading (K) byte
// offset 128 between the two 8-wide channel halves, stride byte offset 256
// between consecutive 8-row groups
__device__ __forceinline__ uint64_t sdesc(uint32_t addr)
{
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

// instruction descriptor: BF16 x BF16 -> FP32, both K-major, M = 128
__host__ __device__ constexpr uint32_t idesc_n(int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc)
{
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
               " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
               "l"(a), "l"(b), "r"(id), "r"(acc)
               : "memory");
}

__device__ __forceinline__ void commit(uint32_t bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16])
{
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int c = 0; c < 16; ++c) v[c] = __uint_as_float(r[c]);
}

__device__ __forceinline__ void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ uint32_t pack2(float lo, float hi)
{
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// Packed FP32 pairs: two independent round-to-nearest operations in one
// instruction, bit for bit the scalar operations.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c)
{
  float2 d;
  asm("{\n .reg .b64 ra, rb, rc, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n mov.b64 rc, {%6, %7};\n"
      " fma.rn.f32x2 rd, ra, rb, rc;\n mov.b64 {%0, %1}, rd;\n}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}

__device__ __forceinline__ float2 mul2(float2 a, float2 b)
{
  float2 d;
  asm("{\n .reg .b64 ra, rb, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
      " mul.rn.f32x2 rd, ra, rb;\n mov.b64 {%0, %1}, rd;\n}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}

__device__ __forceinline__ float tanh_approx(float u)
{
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  return t;
}

// Twice the GELU (tanh form) of two values, packed as BF16:
// x (1 + tanh(u)) with u = x (c2 + c3 x^2), c2 = sqrt(2/pi), c3 = 0.044715 c2,
// with the hardware FP32 tanh and the products on packed pairs.  The factor
// 1/2 of GELU is carried by the next layer's weights (halved when they are
// staged; scaling by 2 is exact in BF16, so the products and sums are those
// of GELU itself).  Half-precision tanh would halve the MUFU work, but it
// moves about one activation in eight to the neighbouring BF16 value, which
// the oracle's FP32 GELU does not.
__device__ __forceinline__ uint32_t gelu2_bf16(float a, float b)
{
  const float2 x = make_float2(a, b);
  const float2 p = fma2(make_float2(0.035677408136300125f, 0.035677408136300125f), mul2(x, x),
                        make_float2(0.7978845608028654f, 0.7978845608028654f));
  const float2 u = mul2(x, p);
  const float2 g = fma2(x, make_float2(tanh_approx(u.x), tanh_approx(u.y)), x);
  return pack2(g.x, g.y);
}

// a BF16 value halved (exact for every normal value)
__device__ __forceinline__ uint16_t half_bf16(uint16_t v)
{
  return (uint16_t)(__float_as_uint(__uint_as_float((uint32_t)v << 16) * 0.5f) >> 16);
}

// 16 channels (8 packed BF16 pairs) of one row into an operand buffer
__device__ __forceinline__ void store_row_packed(unsigned char* buf, int row, const uint32_t (&p)[8])
{
  *reinterpret_cast<uint4*>(buf + core_off(row, 0)) = make_uint4(p[0], p[1], p[2], p[3]);
  *reinterpret_cast<uint4*>(buf + core_off(row, 1)) = make_uint4(p[4], p[5], p[6], p[7]);
}

__device__ __forceinline__ void bar_init(uint32_t bar)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
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

// sum over the CTA; the previous call's reads of red are separated from this
// call's writes by the barriers of the element in between
__device__ __forceinline__ float block_sum4(float v, float* red)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  return red[0] + red[1] + red[2] + red[3];
}

// MMAs of tiles t0 .. t1-1 of one layer, issued by one thread: tile t
// accumulates NMAT products of K = 16 into TMEM columns NCOL * (t % RING)
// (RING = 0: NCOL * t) onwards -- A shifted by the tap's (dj, dk) rows, B the
// tap's weight matrix -- then commits to its barrier.  Fully unrolled over the
// taps: every descriptor is a base plus an immediate offset.
template <int NMAT, int BSTRIDE, int NCOL, bool L1>
__device__ __forceinline__ void issue_tiles(uint32_t tmem, uint64_t da, uint64_t db, uint32_t id,
                                            uint32_t bar_t, int t0, int t1, int ring)
{
  fence_after();
#pragma unroll 1
  for (int t = t0; t < t1; ++t) {
    const uint32_t d = tmem + (uint32_t)(NCOL * (ring ? t % ring : t));
    const uint64_t at = da + (uint64_t)(t * 128 * 16 / 8);  // 128 rows = 16 row groups of 16 units
#pragma unroll
    for (int b = 0; b < NMAT; ++b) {
      const int dj = L1 ? b - 1 : b % 3 - 1, dk = L1 ? 0 : b / 3 - 1;
      const int grp = (kLead + kTile0 + 8 * dj + kPlaneRows * dk) / 8;  // 256-byte row groups
      mma(d, at + (uint64_t)(grp * 16), db + (uint64_t)(b * BSTRIDE / 16), id, b > 0 ? 1u : 0u);
    }
    commit(bar_t + 8 * t);
  }
}

// B operands, [n][k] K-major in core matrices: element (n, k) at
// ((n/8)*2 + k/8)*128 + (n%8)*16 + (k%8)*2
__device__ __forceinline__ int wb_off(int n, int k) { return ((n >> 3) * 2 + (k >> 3)) * 128 + (n & 7) * 16 + (k & 7) * 2; }

// UPDATE: the flexible CG's update is applied first, element by element:
// r -= alpha Ap (written back to r, from which the output's Jacobi term then
// reads) and x += alpha p
template <bool UPDATE>
__global__ void __launch_bounds__(kThreads, kCtasPerSm)
k_net_infer_tc5(int64_t Etot, int64_t Efield, const __nv_bfloat16* __restrict__ Wbf, float* r,
                const float* __restrict__ w, const float* __restrict__ invDiag, float* __restrict__ out,
                int normalize, const int* skip, NetUpdate up)
{
  if (skip != nullptr && *skip != 0) return;
  const float alpha = UPDATE ? (float)*up.alpha : 0.f;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* X = smem + kSmX;
  unsigned char* Y = smem + kSmY;
  float* hs = reinterpret_cast<float*>(smem + kSmH);
  uint16_t* a0 = reinterpret_cast<uint16_t*>(smem + kSmA0);
  float* red = reinterpret_cast<float*>(smem + kSmRed);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint16_t* W = reinterpret_cast<const uint16_t*>(Wbf);
  const uint32_t bar_t = smem_addr(smem + kSmBar);

  // ---- weights as B operands (once per CTA); both activation buffers zeroed
  // (their padding rows are never written again)
  for (int x = tid; x < 3 * 16 * 16; x += kThreads) {  // W1[dj][co][c], c = (di+1) + 3 (dk+1)
    const int a = x / 256, co = (x / 16) % 16, c = x % 16;
    uint16_t v = 0;
    if (c < 9) {
      const int t = (c % 3) + 3 * a + 9 * (c / 3);
      v = W[co * kTaps + t];
    }
    *reinterpret_cast<uint16_t*>(smem + kSmW1 + a * 512 + wb_off(co, c)) = v;
  }
  // layers 2 and 3 take the doubled GELU outputs: their weights are halved
  for (int x = tid; x < 9 * 48 * 16; x += kThreads) {  // W2[(dj,dk)][(di,co)][ci]
    const int b = x / 768, n = (x / 16) % 48, ci = x % 16;
    const int dj = b % 3, dk = b / 3, di = n / 16, co = n % 16;
    const int t = di + 3 * dj + 9 * dk;
    *reinterpret_cast<uint16_t*>(smem + kSmW2 + b * 1536 + wb_off(n, ci)) = half_bf16(W[kO2 + (co * 16 + ci) * kTaps + t]);
  }
  for (int x = tid; x < 9 * 16 * 16; x += kThreads) {  // W3[(dj,dk)][di][ci], di columns 0..2
    const int b = x / 256, n = (x / 16) % 16, ci = x % 16;
    const int dj = b % 3, dk = b / 3;
    uint16_t v = 0;
    if (n < 3) v = half_bf16(W[kO3 + ci * kTaps + n + 3 * dj + 9 * dk]);
    *reinterpret_cast<uint16_t*>(smem + kSmW3 + b * 512 + wb_off(n, ci)) = v;
  }
  for (int x = tid; x < kActBytes / 16; x += kThreads) {
    reinterpret_cast<uint4*>(X)[x] = make_uint4(0, 0, 0, 0);
    reinterpret_cast<uint4*>(Y)[x] = make_uint4(0, 0, 0, 0);
  }
  for (int x = tid; x < kA0Rows * 8 * kA0Rows; x += kThreads) a0[x] = 0;  // its border stays zero
  if (tid == 0) {
    for (int b = 0; b < kTiles; ++b) bar_init(bar_t + 8 * b);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_async_smem();
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + kSmSlot);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *slot;
  const uint32_t tlane = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's TMEM lanes

  // shared-memory descriptors of the operand buffers; an offset of whole
  // 16-byte units is added to the descriptor's start-address field
  const uint64_t dX = sdesc(smem_addr(X)), dY = sdesc(smem_addr(Y));
  const uint64_t dW1 = sdesc(smem_addr(smem + kSmW1)), dW2 = sdesc(smem_addr(smem + kSmW2));
  const uint64_t dW3 = sdesc(smem_addr(smem + kSmW3));
  uint32_t tphase = 0;  // completed phases of every tile barrier
  bool failed = false;
  const int i = lane & 7;  // node i of this thread's rows (tile rows start at multiples of 8)
  auto wait_tile = [&](int t) -> bool {
    const bool ok = bar_wait(bar_t + 8 * t, tphase & 1u);
    fence_after();
    return ok;
  };

  // this thread's residual and diagonal values of the element it starts next
  // (and with UPDATE its A p, p and x values), loaded one element ahead
  // (nodes tid + 128 c)
  float nr[kNp / kThreads], nd[kNp / kThreads], nap[kNp / kThreads], npv[kNp / kThreads],
      nxv[kNp / kThreads];
  auto load_inputs = [&](int64_t el) {
#pragma unroll
    for (int c = 0; c < kNp / kThreads; ++c) {
      const int n = tid + c * kThreads;
      nr[c] = el < Etot ? r[el * kNp + n] : 0.f;
      nd[c] = (el < Etot && invDiag) ? invDiag[(el % Efield) * kNp + n] : 1.f;
      if (UPDATE) {
        nap[c] = el < Etot ? up.Ap[el * kNp + n] : 0.f;
        npv[c] = el < Etot ? up.p[el * kNp + n] : 0.f;
        nxv[c] = el < Etot ? up.x[el * kNp + n] : 0.f;
      }
    }
  };
  load_inputs(blockIdx.x);

  // this thread's tile rows np = kTile0 + 128 t + tid: the node each holds
  // (i, j'-1, k'-1) as a local index and as its centre in the bordered input;
  // rows of the padding lines j' = 0, 9 hold no node (bit t of `live` clear)
  // and are never written after the zeroing above
  int node[kTiles], ctr[kTiles];
  unsigned live = 0;
#pragma unroll
  for (int t = 0; t < kTiles; ++t) {
    const int np = kTile0 + 128 * t + tid;
    const int jp = (np >> 3) % 10, kp = np / kPlaneRows;
    const bool lv = jp >= 1 && jp <= kNq;
    live |= (lv ? 1u : 0u) << t;
    node[t] = lv ? i + kNq * (jp - 1) + kNq * kNq * (kp - 1) : 0;
    ctr[t] = (i + 1) + kA0Rows * (jp - 1) + kA0Plane * kp;
  }

  for (int64_t e = blockIdx.x; e < Etot; e += gridDim.x) {
    const float* rin = r + e * kNp;
    const float* din = invDiag ? invDiag + (e % Efield) * kNp : nullptr;
    const float* win = w ? w + (e % Efield) * kNp : nullptr;

    // ---- scaled input a0 = bf16(h r / s), into the bordered array
    float ss = 0.f, vs[kNp / kThreads];
#pragma unroll
    for (int c = 0; c < kNp / kThreads; ++c) {
      const int n = tid + c * kThreads;
      if (UPDATE) {  // the update pass's r -= alpha Ap and x += alpha p
        nr[c] = fmaf(-alpha, nap[c], nr[c]);
        r[e * kNp + n] = nr[c];
        up.x[e * kNp + n] = fmaf(alpha, npv[c], nxv[c]);
      }
      const float h = din ? sqrtf(nd[c]) : 1.f;
      vs[c] = h * nr[c];
      hs[n] = h;
      ss += vs[c] * vs[c];
    }
    float s = 1.f;
    if (normalize & kNetNormalize) s = sqrtf(block_sum4(ss, red) / kNp);
    const float inv = s > 0.f ? 1.f / s : 0.f;
#pragma unroll
    for (int c = 0; c < kNp / kThreads; ++c) {
      const int n = tid + c * kThreads;
      const __nv_bfloat16 b = __float2bfloat16_rn(vs[c] * inv);
      a0[((n & 7) + 1) + kA0Rows * ((n >> 3) & 7) + kA0Plane * ((n >> 6) + 1)] = *reinterpret_cast<const uint16_t*>(&b);
    }
    __syncthreads();

    // ---- layer-1 operand in X: tile row (i, j', k') holds the 9 inputs at
    // (i + di, j' - 1, k' - 1 + dk), column (di + 1) + 3 (dk + 1), read from
    // the bordered input at offsets di + 80 dk of the node's centre; the other
    // rows keep their zeros (they are layer 3's zero padding)
#pragma unroll
    for (int t = 0; t < kTiles; ++t) {
      if (!((live >> t) & 1u)) continue;
      const uint16_t* q = a0 + ctr[t];
      const int row = kLead + kTile0 + 128 * t + tid;
      *reinterpret_cast<uint4*>(X + core_off(row, 0)) =
          make_uint4(q[-81] | (uint32_t)q[-80] << 16, q[-79] | (uint32_t)q[-1] << 16, q[0] | (uint32_t)q[1] << 16,
                     q[79] | (uint32_t)q[80] << 16);
      *reinterpret_cast<uint4*>(X + core_off(row, 1)) = make_uint4(q[81], 0u, 0u, 0u);
    }
    fence_async_smem();
    fence_before();
    __syncthreads();

    // ---- layer 1: 1 -> 16, GELU, into Y (TMEM columns 16 t)
    if (tid == 0) issue_tiles<3, 512, 16, true>(tmem, dX, dW1, idesc_n(16), bar_t, 0, kTiles, 0);
    bool ok = true;
#pragma unroll 1
    for (int t = 0; t < kTiles; ++t) {
      ok = wait_tile(t) && ok;
      float v[16];
      ld16(tlane + (uint32_t)(16 * t), v);
      ld_wait();
      uint32_t g[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) g[c] = gelu2_bf16(v[2 * c], v[2 * c + 1]);
      if ((live >> t) & 1u) store_row_packed(Y, kLead + kTile0 + 128 * t + tid, g);
    }
    ++tphase;
    fence_async_smem();
    fence_before();
    if (__syncthreads_or(!ok)) { failed = true; break; }

    // ---- layer 2: 16 -> 16, GELU, into X; accumulators in two 48-column
    // buffers (tile t in columns 48 (t % 2))
    if (tid == 0) issue_tiles<9, 1536, 48, false>(tmem, dY, dW2, idesc_n(48), bar_t, 0, 2, 2);
#pragma unroll 1
    for (int t = 0; t < kTiles; ++t) {
      ok = wait_tile(t) && ok;
      float vm[16], v0[16], vp[16];
      const uint32_t col = (uint32_t)(48 * (t & 1));
      ld16(tlane + col, vm);
      ld16(tlane + col + 16, v0);
      ld16(tlane + col + 32, vp);
      ld_wait();
      if (t + 2 < kTiles) {  // every warp has read buffer t % 2: reuse it for tile t + 2
        fence_before();
        __syncthreads();
        if (tid == 0) issue_tiles<9, 1536, 48, false>(tmem, dY, dW2, idesc_n(48), bar_t, t + 2, t + 3, 2);
      }
      // out(i) = V(i)[0] + V(i + 1)[+1] + V(i - 1)[-1], the neighbours' terms
      // taken inside the element only (a factor 1 or 0: 1 x + o rounds as o + x)
      const float2 fu = make_float2(i < kNq - 1 ? 1.f : 0.f, i < kNq - 1 ? 1.f : 0.f);
      const float2 fd = make_float2(i > 0 ? 1.f : 0.f, i > 0 ? 1.f : 0.f);
#pragma unroll
      for (int c = 0; c < 16; c += 2) {
        const float2 up = make_float2(__shfl_down_sync(0xffffffffu, vp[c], 1),  // node i + 1, column di = +1
                                      __shfl_down_sync(0xffffffffu, vp[c + 1], 1));
        const float2 dn = make_float2(__shfl_up_sync(0xffffffffu, vm[c], 1),  // node i - 1, column di = -1
                                      __shfl_up_sync(0xffffffffu, vm[c + 1], 1));
        const float2 o = fma2(dn, fd, fma2(up, fu, make_float2(v0[c], v0[c + 1])));
        v0[c] = o.x;
        v0[c + 1] = o.y;
      }
      uint32_t g[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) g[c] = gelu2_bf16(v0[2 * c], v0[2 * c + 1]);
      if ((live >> t) & 1u) store_row_packed(X, kLead + kTile0 + 128 * t + tid, g);
    }
    ++tphase;
    fence_async_smem();
    fence_before();
    if (__syncthreads_or(!ok)) { failed = true; break; }

    // ---- layer 3: 16 -> 1 and the output (TMEM columns 16 t)
    if (tid == 0) issue_tiles<9, 512, 16, false>(tmem, dX, dW3, idesc_n(16), bar_t, 0, kTiles, 0);
    // the output's inputs for this thread's five rows, and the next element's
    // residual and diagonal, requested before the MMAs are waited for
    float ojac[kTiles], ow[kTiles];
#pragma unroll
    for (int t = 0; t < kTiles; ++t) {
      const int n = node[t];
      ojac[t] = ((normalize & kNetAddJacobi) && din) ? din[n] * rin[n] : 0.f;
      ow[t] = win ? win[n] : 1.f;
    }
    load_inputs(e + gridDim.x);
#pragma unroll
    for (int t = 0; t < kTiles; ++t) {
      ok = wait_tile(t) && ok;
      float v[16];
      ld16(tlane + (uint32_t)(16 * t), v);
      ld_wait();
      const float up = __shfl_down_sync(0xffffffffu, v[2], 1);
      const float dn = __shfl_up_sync(0xffffffffu, v[0], 1);
      float o = v[1];
      if (i < kNq - 1) o += up;
      if (i > 0) o += dn;
      if ((live >> t) & 1u) {
        const int n = node[t];
        out[e * kNp + n] = ow[t] * (o * (hs[n] * s) + ojac[t]);
      }
    }
    ++tphase;
    fence_before();
    if (__syncthreads_or(!ok)) { failed = true; break; }
  }

  if (failed) {  // flag, then wait (bounded) for this CTA's MMAs in flight
    if (tid == 0) {
      atomicExch(&g_tc5_timeout, 1);
      for (int t = 0; t < kTiles; ++t) bar_wait(bar_t + 8 * t, (tphase - 1u) & 1u);  // the layer that stopped
    }
    fence_before();
    __syncthreads();
  }
  fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

}  // namespace

// reads and clears the timeout flag
int net_tc5_take_timeout(int* flag)
{
  NEKB_CUDA(cudaMemcpyFromSymbol(flag, g_tc5_timeout, sizeof(int)));
  if (*flag) {
    const int zero = 0;
    NEKB_CUDA(cudaMemcpyToSymbol(g_tc5_timeout, &zero, sizeof(int)));
  }
  return NEKB_OK;
}

int net_tc5_raise_timeout()
{
  const int one = 1;
  NEKB_CUDA(cudaMemcpyToSymbol(g_tc5_timeout, &one, sizeof(int)));
  return NEKB_OK;
}

int net_infer_tc5(const __nv_bfloat16* Wbf, int64_t Etot, int64_t Efield, const float* r, const float* w,
                  const float* invDiag, float* out, int normalize, const int* skip, cudaStream_t s,
                  const NetUpdate* up)
{
  static SmemOptIn smem_plain, smem_update;
  if (up) {
    NEKB_TRY(smem_update.ensure(k_net_infer_tc5<true>, kSmTotal));
  } else {
    NEKB_TRY(smem_plain.ensure(k_net_infer_tc5<false>, kSmTotal));
  }
  int dev = 0, sms = 152;
  NEKB_CUDA(cudaGetDevice(&dev));
  NEKB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // kCtasPerSm CTAs fit an SM by construction (the static_asserts above); the
  // occupancy query is not used, as it reported one CTA per SM for a kernel
  // of which two fit
  int64_t grid = (int64_t)sms * kCtasPerSm;
  if (grid > Etot) grid = Etot;
  if (grid < 1) return NEKB_OK;
  // r is written only with the update, which the caller passes a writable r for
  float* rw = const_cast<float*>(r);
  if (up)
    k_net_infer_tc5<true><<<(unsigned)grid, kThreads, kSmTotal, s>>>(Etot, Efield, Wbf, rw, w, invDiag, out,
                                                                     normalize, skip, *up);
  else
    k_net_infer_tc5<false><<<(unsigned)grid, kThreads, kSmTotal, s>>>(Etot, Efield, Wbf, rw, w, invDiag,
                                                                      out, normalize, skip, NetUpdate{});
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

}  // namespace nekb
