// Internal declarations shared by the translation units of libnekb_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <atomic>
#include <cstdint>
#include <vector>

#include "nekb.h"

namespace nekb {

// ---------------------------------------------------------------- errors
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);
void clear_error();

#define NEKB_CUDA(call)                                                         \
  do {                                                                          \
    cudaError_t nekb_e_ = (call);                                               \
    if (nekb_e_ != cudaSuccess) return ::nekb::cuda_fail(nekb_e_, #call, __FILE__, __LINE__); \
  } while (0)

#define NEKB_TRY(call)                  \
  do {                                  \
    int nekb_s_ = (call);               \
    if (nekb_s_ != NEKB_OK) return nekb_s_; \
  } while (0)

// Opt-in of one kernel to more than 48 KB of dynamic shared memory.  The
// attribute belongs to each device's context, so it is set once per device
// (ordinals 0..63 are remembered; beyond that it is set at every launch).  The
// solvers launch every operator once before they capture a graph, so the
// first launch on a device never falls inside a capture.
struct SmemOptIn {
  std::atomic<uint64_t> done{0};
  template <typename K>
  int ensure(K kern, int bytes)
  {
    int dev = 0;
    NEKB_CUDA(cudaGetDevice(&dev));
    const uint64_t bit = (dev >= 0 && dev < 64) ? (uint64_t(1) << dev) : 0;
    if (bit != 0 && (done.load(std::memory_order_acquire) & bit) != 0) return 0;
    NEKB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    done.fetch_or(bit, std::memory_order_release);
    return 0;
  }
};

constexpr int kMaxNq = 14;      // FP64; the other precisions go to kMaxNqReduced
constexpr int kMaxNqReduced = 12;
constexpr int kMinNq = 2;

// ---------------------------------------------------------------- basis (host)
int gll_nodes(int N, double* r, double* w);
int gauss_nodes(int N, double* r, double* w);
void deriv_matrix(int Nq, const double* r, double* D);

// ---------------------------------------------------------------- random numbers
__host__ __device__ inline uint64_t mix64(uint64_t x)
{
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__host__ __device__ inline double uniform01(uint64_t seed, uint64_t stream, uint64_t i)
{
  const uint64_t h = mix64(mix64(seed * 0xD1B54A32D192ED03ull + stream) + i);
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------- axhelm
struct AxArgs {
  int64_t Nelements;
  int64_t offset;
  const int32_t* elementList;
  const void* ggeo;     // ggeo (double/float/bf16) or trilinear coefficients (float [E][24])
  const void* D;        // double (FP64) or float
  const void* lambda;   // same type as ggeo storage for BF16, else compute type; may be null for BK
  const void* q;
  void* Aq;
  const int* skip;      // optional device flag: kernel returns at once when *skip != 0
  // optional: per-block sums of q . Aq (local, before assembly) into
  // dot_partials[block], the block count into *dot_count (non-Partial forms)
  double* dot_partials;
  int* dot_count;
  float r1d[kMaxNq];    // GLL nodes and weights (trilinear geometry only)
  float w1d[kMaxNq];
};

int launch_axhelm(int Nq, int flags, int precision, const AxArgs& a, cudaStream_t s);

int launch_update_jacobi(int Nq, int64_t E, int64_t offset, const int32_t* mapB, const double* ggeo,
                         const double* D, const double* lambda, int bk, double* diag,
                         cudaStream_t s);
int launch_geometric_factors(int Nq, int64_t E, const double* EX, const double* EY,
                             const double* EZ, const double* r1d, const double* w1d, double* ggeo,
                             cudaStream_t s);
int launch_trilinear_coeffs(int64_t E, const double* EX, const double* EY, const double* EZ,
                            float* coef, cudaStream_t s);
int launch_physical_nodes(int Nq, int64_t E, const double* EX, const double* EY, const double* EZ,
                          const double* r1d, double* x, double* y, double* z, cudaStream_t s);

// ---------------------------------------------------------------- gather-scatter
// gatherScatterMany add over the multi-member groups of `ogs` (k fields of the
// given stride)
int launch_gs_add(const nekb_ogs* ogs, int k, int64_t stride, void* q, int dtype, const int* skip,
                  cudaStream_t s);
int launch_mask(int64_t Nmasked, const int32_t* ids, int k, int64_t stride, void* q, int dtype,
                const int* skip, cudaStream_t s);

// ---------------------------------------------------------------- vector kernels
int launch_fill_uniform(double* v, int64_t n, uint64_t seed, uint64_t stream, double lo, double hi,
                        cudaStream_t s);
int launch_convert_d2f(const double* a, float* b, int64_t n, cudaStream_t s);
int launch_convert_d2bf(const double* a, __nv_bfloat16* b, int64_t n, cudaStream_t s);
int launch_scale(double* v, double alpha, int64_t n, cudaStream_t s);
int launch_vec_inv(double* v, int64_t n, cudaStream_t s);
int launch_set_scalar(double* v, double alpha, int64_t n, cudaStream_t s);

}  // namespace nekb

// ---------------------------------------------------------------- handles
struct nekb_ogs {
  int64_t N = 0;
  int64_t Nlocal = 0;
  int64_t NlocalGather = 0;
  int64_t Nmulti = 0;                 // groups with more than one member
  std::vector<int32_t> h_offsets;     // NlocalGather+1 (reference CSR, host)
  std::vector<int32_t> h_ids;         // Nlocal
  // device copy of the multi-member groups, cut in CSR order into chunks of
  // kGsChunk groups and, within a chunk, by size: groups of two and of four
  // as packed member ids (a box mesh's face and edge nodes), every other size
  // as CSR; members in CSR order within each group
  static constexpr int kGsChunk = 2048;
  int64_t Npairs = 0, Nquads = 0, Nrest = 0, Nchunks = 0;
  int32_t* d_chunks = nullptr;        // 3 (Nchunks+1): first pair, quad, other group of each chunk
  int32_t* d_pairs = nullptr;         // 2 Npairs
  int32_t* d_quads = nullptr;         // 4 Nquads
  int32_t* d_offsets = nullptr;       // Nrest+1
  int32_t* d_ids = nullptr;           // members of the other groups
  double* d_invDegree = nullptr;      // N
};
