// Weighted inner product that allocates no device memory.
//
// Some callers cannot call cudaMalloc: an application that has handed all of
// the GPU's memory to its own pool allocator (a raw cudaMalloc then fails, or
// fragments the pool behind the allocator's back), or a time-critical loop
// that must not trigger the implicit device synchronisation cudaMalloc can
// cause.  For them this entry point keeps its scratch -- one partial sum per
// 256-node block and a block-completion ticket -- in a fixed array compiled
// into the library, so a call needs only the caller's inputs and output.
#include <mutex>

#include "internal.h"

namespace nekb {
int launch_wdot(int64_t N, int NF, int64_t offset, const double* w, const double* u,
                const double* v, bool two, int64_t grid, double* partials, unsigned* counter,
                double* out, cudaStream_t s);
}  // namespace nekb

namespace {

// 2^17 partial sums: 1 MiB, enough for 2^17 * 256 = 33,554,432 nodes per field.
constexpr int64_t kNoAllocBlocks = int64_t(1) << 17;
constexpr int64_t kNoAllocMaxNodes = kNoAllocBlocks * 256;
constexpr int kMaxDevices = 64;

// Partials in [0, kNoAllocBlocks), the ticket counter in the first word after
// them.  Every GPU that loads the library holds this array until the process
// exits; every call shares it.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocBlocks + 32];

std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Device address of the array on the current device, looked up once per
// device (the host-side symbol is only a stand-in, never a device address).
int scratch_address(double** out)
{
  int dev = 0;
  NEKB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return nekb::fail(NEKB_ERR_UNSUPPORTED, "no-alloc inner product: device %d beyond %d", dev,
                      kMaxDevices);
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_addr[dev] == nullptr) {
    void* p = nullptr;
    NEKB_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_addr[dev] = p;
  }
  *out = static_cast<double*>(g_addr[dev]);
  return NEKB_OK;
}

}  // namespace

extern "C" int nekb_weighted_inner_product_noalloc(int64_t N, int Nfields, int64_t offset,
                                                   const double* w, const double* a,
                                                   const double* b, double* wab, void* stream)
{
  using namespace nekb;
  if (N < 0 || Nfields < 1 || Nfields > 3 || (Nfields > 1 && offset < N))
    return fail(NEKB_ERR_INVALID, "no-alloc inner product: N=%lld Nfields=%d offset=%lld",
                (long long)N, Nfields, (long long)offset);
  if (N > kNoAllocMaxNodes)
    return fail(NEKB_ERR_INVALID,
                "no-alloc inner product: N=%lld nodes per field exceeds the fixed scratch "
                "(at most %lld nodes per field)", (long long)N, (long long)kNoAllocMaxNodes);
  if (!wab || (N > 0 && (!w || !a || !b)))
    return fail(NEKB_ERR_INVALID, "no-alloc inner product: NULL argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (N == 0) {
    NEKB_CUDA(cudaMemsetAsync(wab, 0, sizeof(double), s));
    return NEKB_OK;
  }
  double* scratch = nullptr;
  NEKB_TRY(scratch_address(&scratch));
  unsigned* ticket = reinterpret_cast<unsigned*>(scratch + kNoAllocBlocks);
  // the ticket must start at zero; the previous call leaves it at zero, but a
  // call that failed part-way might not have
  NEKB_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned), s));
  const int64_t grid = (N + 255) / 256;
  return launch_wdot(N, Nfields, offset, w, a, b, false, grid, scratch, ticket, wab, s);
}
