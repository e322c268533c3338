// Per-block partial sums of the dot benchmark (dot/kernel/VOLTA/dot.okl):
//   variant 0  weightedInnerProduct2_v0   (dot.okl:27-65)   blocks of 256, 512 or 1024 nodes
//   variant 1  weightedInnerProduct2_v1   (dot.okl:114-169) blocks of 256 = 8 groups of 32
//   variant 2  weightedBlockInnerProduct2 (dot.okl:67-111)  v0's tree over a per-node sum of
//              Nfields triple products, w indexed per field like x and y
// The driver sums the partials on the host in block order (dot/main.cpp:27-48).
//
// One warp reduces one reference block of B nodes: lane l holds the products
// of nodes l + 32 m, m < B / 32, loaded with 256-byte coalesced accesses.  The
// reference halves its shared array (s[t] += s[t + h] for t < h, h = B/2, ...,
// 2, then s[0] + s[1]); for h >= 32 both operands of every addition sit in the
// same lane (registers m and m + h/32), for h <= 16 they are h lanes apart and
// come through a shuffle.  So every addition is the reference's own, in its
// order, and the partials match the reference tree bit for bit.  Products are
// rounded with __dmul_rn so that no multiply-add is contracted.
//
// variant 1 reduces each group of 32 nodes with the in-warp steps h = 16, 8, 4,
// 2 and s[0] + s[1], then the 8 group sums with h = 4, 2, 1.  The reference
// kernel issues those steps with no barrier between them, so its result relies
// on the 32 threads of a group running in lockstep; this is the lockstep tree.
#include "internal.h"

namespace nekb {
namespace {

constexpr int kWarpsPerCta = 8;

// product (or per-node sum over fields) at node id, 0 beyond N
template <int VARIANT>
__device__ __forceinline__ double node_value(int64_t id, int64_t N, int NF, int64_t offset,
                                             const double* __restrict__ w,
                                             const double* __restrict__ x,
                                             const double* __restrict__ y)
{
  if (VARIANT == 2) {
    double res = 0.0;
    if (id < N)
      for (int f = 0; f < NF; ++f) {
        const int64_t k = id + f * offset;
        res = __dadd_rn(res, __dmul_rn(__dmul_rn(w[k], x[k]), y[k]));
      }
    return res;
  }
  return id < N ? __dmul_rn(__dmul_rn(w[id], x[id]), y[id]) : 0.0;
}

template <int VARIANT, int J>  // J = B / 32 values per lane
__global__ void __launch_bounds__(32 * kWarpsPerCta)
k_dot_partials(int64_t N, int NF, int64_t offset, int64_t nblock, const double* __restrict__ w,
               const double* __restrict__ x, const double* __restrict__ y,
               double* __restrict__ wxy)
{
  const int lane = threadIdx.x & 31;
  const int64_t b = (int64_t)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  if (b >= nblock) return;  // whole warps leave together
  const int64_t base = b * (32 * J) + lane;
  double v[J];
#pragma unroll
  for (int m = 0; m < J; ++m) v[m] = node_value<VARIANT>(base + 32 * m, N, NF, offset, w, x, y);

  if (VARIANT == 1) {
    // groups m = 0..7: in-group steps 16, 8, 4, 2 then s[0] + s[1]
#pragma unroll
    for (int h = 16; h >= 2; h >>= 1)
#pragma unroll
      for (int m = 0; m < J; ++m) v[m] += __shfl_down_sync(0xffffffffu, v[m], h);
#pragma unroll
    for (int m = 0; m < J; ++m) v[m] += __shfl_down_sync(0xffffffffu, v[m], 1);
    if (lane == 0) {
#pragma unroll
      for (int h = J / 2; h >= 1; h >>= 1)
#pragma unroll
        for (int m = 0; m < h; ++m) v[m] += v[m + h];
      wxy[b] = v[0];
    }
    return;
  }
  // steps h = B/2 .. 32: registers m and m + h/32 of the same lane
#pragma unroll
  for (int hm = J / 2; hm >= 1; hm >>= 1)
#pragma unroll
    for (int m = 0; m < hm; ++m) v[m] += v[m + hm];
  double s = v[0];
  // steps h = 16 .. 2 across lanes, then s[0] + s[1]
#pragma unroll
  for (int h = 16; h >= 2; h >>= 1) s += __shfl_down_sync(0xffffffffu, s, h);
  const double s1 = __shfl_down_sync(0xffffffffu, s, 1);
  if (lane == 0) wxy[b] = s + s1;
}

template <int VARIANT, int J>
int launch(int64_t N, int NF, int64_t offset, int64_t nblock, const double* w, const double* x,
           const double* y, double* wxy, cudaStream_t s)
{
  const int64_t grid = (nblock + kWarpsPerCta - 1) / kWarpsPerCta;
  if (grid > INT32_MAX) return fail(NEKB_ERR_INVALID, "dot: %lld blocks", (long long)nblock);
  k_dot_partials<VARIANT, J><<<(unsigned)grid, 32 * kWarpsPerCta, 0, s>>>(N, NF, offset, nblock, w, x,
                                                                          y, wxy);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

}  // namespace
}  // namespace nekb

extern "C" int64_t nekb_dot_num_blocks(int64_t N, int blockSize)
{
  if (N < 0 || (blockSize != 256 && blockSize != 512 && blockSize != 1024))
    return nekb::fail(NEKB_ERR_INVALID, "dot: N=%lld blockSize %d", (long long)N, blockSize);
  return (N + blockSize - 1) / blockSize;
}

extern "C" int nekb_dot_partials(int variant, int64_t N, int Nfields, int64_t offset, int blockSize,
                                 const double* w, const double* x, const double* y, double* wxy,
                                 void* stream)
{
  using namespace nekb;
  if (variant < 0 || variant > 2)
    return fail(NEKB_ERR_INVALID, "dot: variant %d (0 = v0, 1 = v1, 2 = block)", variant);
  if (blockSize != 256 && blockSize != 512 && blockSize != 1024)
    return fail(NEKB_ERR_INVALID, "dot: blockSize %d (256, 512 or 1024)", blockSize);
  if (variant == 1 && blockSize != 256)
    return fail(NEKB_ERR_INVALID, "dot: weightedInnerProduct2_v1 reduces blocks of 256 nodes");
  const int NF = variant == 2 ? Nfields : 1;
  if (N < 0 || NF < 1 || NF > 3 || (NF > 1 && offset < N))
    return fail(NEKB_ERR_INVALID, "dot: N=%lld Nfields=%d offset=%lld", (long long)N, Nfields,
                (long long)offset);
  if (variant == 1 && N > INT32_MAX)
    return fail(NEKB_ERR_INVALID, "dot: weightedInnerProduct2_v1 takes an int node count");
  if (N == 0) return NEKB_OK;
  if (!w || !x || !y || !wxy) return fail(NEKB_ERR_INVALID, "dot: NULL argument");
  const int64_t nblock = (N + blockSize - 1) / blockSize;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (variant == 1) return launch<1, 8>(N, 1, 0, nblock, w, x, y, wxy, s);
  if (variant == 0) {
    if (blockSize == 256) return launch<0, 8>(N, 1, 0, nblock, w, x, y, wxy, s);
    if (blockSize == 512) return launch<0, 16>(N, 1, 0, nblock, w, x, y, wxy, s);
    return launch<0, 32>(N, 1, 0, nblock, w, x, y, wxy, s);
  }
  if (blockSize == 256) return launch<2, 8>(N, NF, offset, nblock, w, x, y, wxy, s);
  if (blockSize == 512) return launch<2, 16>(N, NF, offset, nblock, w, x, y, wxy, s);
  return launch<2, 32>(N, NF, offset, nblock, w, x, y, wxy, s);
}
