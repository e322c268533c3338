// nekBone PCG on the device (BPPCG, nekBone/solve.cpp:44-113) and its mixed
// precision form.
//
// All scalars (rdotz, rdotr, alpha, beta, TOL, the iteration counter and the
// convergence flag) live in device memory and are updated by the last block
// of each reduction, so an iteration needs no host round trip; the host reads
// the state once per chunk of iterations, and each chunk is replayed as a
// CUDA graph.  Kernels after convergence see the flag and return at once.
//
// Reductions are deterministic: fixed grid, fixed per-thread order, fixed
// tree, and the final sum over block partials in block order.
//
// Per iteration (reference order, solve.cpp:76-109):
//   K_p   : p = z + beta p                          (BPScaledAdd)
//   axhelm, gather-scatter, mask : Ap = A p          (BPAxOperator)
//   K_pAp : pAp = sum w p Ap ; alpha = rdotz/pAp     (BPWeightedInnerProduct)
//   K_upd : x += alpha p ; r -= alpha Ap ; z = M r ; (BPUpdatePCG fused with
//           rdotz = sum w r z ; rdotr = sum w r r     BPPreconditioner and
//           convergence test, beta                     BPWeightedInnerProduct2)
// In the FP32 inner iterations K_pAp is replaced by the operator kernel's own
// per-block sums of p . A_local p and a one-block reduction.  With the learned
// preconditioner the iteration is truncated flexible CG, FCG(m): the new
// direction is z minus its A-projections on the last m directions (ring
// buffers), alpha = r.p / p.Ap.
#include "bp.h"
#include "nn.h"

#include <cmath>
#include <cstring>
#include <functional>

namespace nekb {

namespace {

constexpr int RT = 256;           // threads per reduction block
constexpr int kMaxRedBlocks = 1216;  // 152 SMs x 8 resident blocks

enum { PC_COPY = 0, PC_JACOBI = 1, PC_EXTERNAL = 2 };

template <typename T>
struct PcgArgs {
  int64_t Nloc;
  int64_t offset;
  int NF;
  const T* w;        // invDegree (Nloc)
  const T* invDiag;  // Jacobi (Nloc) or null
  T* r;
  T* x;
  T* p;
  T* z;
  T* Ap;
  PcgState* st;
  double* partials;
  unsigned* counter;
  double* out;       // k_wdot result
};

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// block sum of NV values; the result is valid in thread 0
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double (*sh)[RT / 32])
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    v[k] = warp_sum(v[k]);
    if (lane == 0) sh[k][warp] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = lane < RT / 32 ? sh[k][lane] : 0.0;
      v[k] = warp_sum(t);
    }
  }
  __syncthreads();
}

// block partial -> partials[k*gridDim + b]; returns true in the last block,
// whose thread 0 then holds the totals in v (summed in block order).
template <int NV>
__device__ bool grid_sum(double (&v)[NV], double* partials, unsigned* counter)
{
  __shared__ double sh[NV][RT / 32];
  __shared__ unsigned s_last;
  block_sum<NV>(v, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
    __threadfence();
    s_last = (atomicAdd(counter, 1u) == gridDim.x - 1) ? 1u : 0u;
  }
  __syncthreads();
  if (s_last == 0) return false;
  __threadfence();
  double t[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) t[k] = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += RT)
#pragma unroll
    for (int k = 0; k < NV; ++k) t[k] += __ldcg(&partials[k * gridDim.x + b]);
  block_sum<NV>(t, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = t[k];
    *counter = 0u;
  }
  return threadIdx.x == 0;
}

// convergence test and beta after the (r,z) inner products (solve.cpp:77-98)
__device__ void state_after_rz(PcgState* st, double rz, double rr, double zAp)
{
  const int it = ++st->iter;
  if (it > st->maxit) {
    st->done = 1;
    st->result = st->maxit;
    if (!st->fixed) st->status = NEKB_ERR_NOT_CONVERGED;
    return;
  }
  st->rdotz2 = st->rdotz1;
  st->rdotz1 = rz;
  st->rdotr = rr;
  if (it == 1) {
    st->rdotr0 = rr;
    st->TOL = fmax(st->tol2 * rr, st->tol2);
  }
  if (rr <= st->TOL && !st->fixed) {
    st->done = 1;
    st->result = it - 1;
    return;
  }
  double beta;
  if (st->flexible)
    beta = -st->alpha * zAp / st->rdotz2;
  else
    beta = (it == 1) ? 0.0 : st->rdotz1 / st->rdotz2;
  if (!isfinite(beta) || !isfinite(rr)) {
    st->done = 1;
    st->result = it - 1;
    st->status = NEKB_ERR_BREAKDOWN;
    return;
  }
  st->zdotAp = zAp;
  st->beta = beta;
}

// after the residual was replaced by the true one: new rdotz and beta, same
// iteration (the search direction p is kept)
__device__ void state_refresh(PcgState* st, double rz, double rr, double zAp)
{
  st->rdotz1 = rz;
  st->rdotr = rr;
  double beta;
  if (st->flexible)
    beta = -st->alpha * zAp / st->rdotz2;
  else
    beta = (st->iter <= 1) ? 0.0 : rz / st->rdotz2;
  if (!isfinite(beta) || !isfinite(rr)) {
    st->done = 1;
    st->result = st->iter - 1;
    st->status = NEKB_ERR_BREAKDOWN;
    return;
  }
  st->zdotAp = zAp;
  st->beta = beta;
}

// V consecutive entries per access: V = 4 (float4) for FP32 vectors whose
// length and field offset are multiples of 4, else 1
template <int V, typename T>
__device__ __forceinline__ void vld(const T* p, T (&v)[V])
{
  if constexpr (V == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  } else {
    v[0] = *p;
  }
}
template <int V, typename T>
__device__ __forceinline__ void vst(T* p, const T (&v)[V])
{
  if constexpr (V == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
    *p = v[0];
  }
}

// [x += alpha p; r -= alpha Ap;] z = M r; sums w r z, w r r (, w z Ap)
template <typename T, int MODE, bool UPDATE, bool FLEX, bool REFRESH = false, int V = 1>
__global__ void __launch_bounds__(RT) k_update_rz(PcgArgs<T> a)
{
  PcgState* st = a.st;
  if (st->done) return;
  const T alpha = UPDATE ? (T)st->alpha : T(0);
  T rz = 0, rr = 0, za = 0;
  const int64_t stride = (int64_t)gridDim.x * RT;
  const int64_t nv = a.Nloc / V;
  for (int f = 0; f < a.NF; ++f) {
    const int64_t fo = f * a.offset;
    for (int64_t iv = (int64_t)blockIdx.x * RT + threadIdx.x; iv < nv; iv += stride) {
      const int64_t i = iv * V, n = i + fo;
      T r[V], ap[V], z[V], w[V];
      vld<V>(a.r + n, r);
      if (UPDATE || FLEX) vld<V>(a.Ap + n, ap);
      if (UPDATE) {
        T x[V], p[V];
        vld<V>(a.x + n, x);
        vld<V>(a.p + n, p);
#pragma unroll
        for (int l = 0; l < V; ++l) {
          x[l] += alpha * p[l];
          r[l] -= alpha * ap[l];
        }
        vst<V>(a.x + n, x);
        vst<V>(a.r + n, r);
      }
      if (MODE == PC_COPY) {
#pragma unroll
        for (int l = 0; l < V; ++l) z[l] = r[l];
      } else if (MODE == PC_JACOBI) {
        T d[V];
        vld<V>(a.invDiag + i, d);
#pragma unroll
        for (int l = 0; l < V; ++l) z[l] = d[l] * r[l];
        vst<V>(a.z + n, z);
      } else {
        vld<V>(a.z + n, z);
      }
      vld<V>(a.w + i, w);
#pragma unroll
      for (int l = 0; l < V; ++l) {
        rz += w[l] * r[l] * z[l];
        rr += w[l] * r[l] * r[l];
        if (FLEX) za += w[l] * z[l] * ap[l];
      }
    }
  }
  double v[3] = {(double)rz, (double)rr, (double)za};
  if (grid_sum<3>(v, a.partials, a.counter)) {
    if (REFRESH)
      state_refresh(st, v[0], v[1], v[2]);
    else
      state_after_rz(st, v[0], v[1], v[2]);
  }
}

// x += alpha p ; r -= alpha Ap (external preconditioner path)
template <typename T>
__global__ void __launch_bounds__(RT) k_update(PcgArgs<T> a)
{
  if (a.st->done) return;
  const T alpha = (T)a.st->alpha;
  const int64_t N = a.NF * a.offset;
  for (int64_t n = (int64_t)blockIdx.x * RT + threadIdx.x; n < N; n += (int64_t)gridDim.x * RT) {
    a.x[n] += alpha * a.p[n];
    a.r[n] -= alpha * a.Ap[n];
  }
}

// p = z + beta p   (z = r for the COPY preconditioner)
template <typename T, int MODE, int V = 1>
__global__ void __launch_bounds__(RT) k_pupdate(PcgArgs<T> a)
{
  if (a.st->done) return;
  const T beta = (T)a.st->beta;
  const T* zs = (MODE == PC_COPY) ? a.r : a.z;
  const int64_t N = a.NF * a.offset / V;
  for (int64_t nv = (int64_t)blockIdx.x * RT + threadIdx.x; nv < N; nv += (int64_t)gridDim.x * RT) {
    T z[V], p[V];
    vld<V>(zs + nv * V, z);
    vld<V>(a.p + nv * V, p);
#pragma unroll
    for (int l = 0; l < V; ++l) p[l] = z[l] + beta * p[l];
    vst<V>(a.p + nv * V, p);
  }
}

// ---- truncated flexible CG, FCG(m), for the external (learned) preconditioner.
// The last m directions p_j and A p_j sit in ring slots (stride `ring`
// entries); the new direction is z minus its A-projections on them,
//   p = z - sum_j (z . A p_j / p_j . A p_j) p_j ,  alpha = r . p / p . A p .

// (r, z) sums and z . A p_j for the kept directions; REFRESH: same iteration
template <typename T, int V, bool REFRESH>
__global__ void __launch_bounds__(RT) k_fcg_dots(PcgArgs<T> a, const T* __restrict__ AP, int64_t ring)
{
  PcgState* st = a.st;
  if (st->done) return;
  const int cnt = st->fcg_count;
  T rz = 0, rr = 0, zap[kFcgMax];
#pragma unroll
  for (int j = 0; j < kFcgMax; ++j) zap[j] = 0;
  const int64_t stride = (int64_t)gridDim.x * RT;
  const int64_t nv = a.Nloc / V;
  for (int f = 0; f < a.NF; ++f) {
    const int64_t fo = f * a.offset;
    for (int64_t iv = (int64_t)blockIdx.x * RT + threadIdx.x; iv < nv; iv += stride) {
      const int64_t i = iv * V, n = i + fo;
      T r[V], z[V], w[V];
      vld<V>(a.r + n, r);
      vld<V>(a.z + n, z);
      vld<V>(a.w + i, w);
#pragma unroll
      for (int l = 0; l < V; ++l) {
        rz += w[l] * r[l] * z[l];
        rr += w[l] * r[l] * r[l];
      }
#pragma unroll
      for (int j = 0; j < kFcgMax; ++j) {
        if (j < cnt) {
          T ap[V];
          vld<V>(AP + j * ring + n, ap);
#pragma unroll
          for (int l = 0; l < V; ++l) zap[j] += w[l] * z[l] * ap[l];
        }
      }
    }
  }
  double v[2 + kFcgMax];
  v[0] = (double)rz;
  v[1] = (double)rr;
#pragma unroll
  for (int j = 0; j < kFcgMax; ++j) v[2 + j] = (double)zap[j];
  if (grid_sum<2 + kFcgMax>(v, a.partials, a.counter)) {
    if (REFRESH)
      state_refresh(st, v[0], v[1], 0.0);
    else
      state_after_rz(st, v[0], v[1], 0.0);
#pragma unroll
    for (int j = 0; j < kFcgMax; ++j) st->fcg_zap[j] = v[2 + j];
  }
}

// p = z - sum_j c_j p_j into the operator's p and into the ring slot `head`
template <typename T, int V>
__global__ void __launch_bounds__(RT) k_fcg_pupdate(PcgArgs<T> a, T* __restrict__ P, int64_t ring)
{
  const PcgState* st = a.st;
  if (st->done) return;
  const int cnt = st->fcg_count, head = st->fcg_head;
  T c[kFcgMax];
#pragma unroll
  for (int j = 0; j < kFcgMax; ++j)
    c[j] = (j < cnt && st->fcg_pap[j] > 0.0) ? (T)(st->fcg_zap[j] / st->fcg_pap[j]) : T(0);
  const int64_t N = a.NF * a.offset / V;
  for (int64_t nv = (int64_t)blockIdx.x * RT + threadIdx.x; nv < N; nv += (int64_t)gridDim.x * RT) {
    T p[V];
    vld<V>(a.z + nv * V, p);
#pragma unroll
    for (int j = 0; j < kFcgMax; ++j) {
      if (j < cnt) {
        T pj[V];
        vld<V>(P + j * ring + nv * V, pj);
#pragma unroll
        for (int l = 0; l < V; ++l) p[l] -= c[j] * pj[l];
      }
    }
    vst<V>(a.p + nv * V, p);
    vst<V>(P + head * ring + nv * V, p);
  }
}

// pAp = sum w p Ap, rp = sum w r p; alpha = rp / pAp; A p into the ring slot;
// the slot becomes a kept direction
template <typename T, int V>
__global__ void __launch_bounds__(RT) k_fcg_pap(PcgArgs<T> a, T* __restrict__ AP, int64_t ring)
{
  PcgState* st = a.st;
  if (st->done) return;
  const int head = st->fcg_head;
  T pap = 0, rp = 0;
  const int64_t stride = (int64_t)gridDim.x * RT;
  const int64_t nv = a.Nloc / V;
  for (int f = 0; f < a.NF; ++f) {
    const int64_t fo = f * a.offset;
    for (int64_t iv = (int64_t)blockIdx.x * RT + threadIdx.x; iv < nv; iv += stride) {
      const int64_t i = iv * V, n = i + fo;
      T w[V], p[V], ap[V], r[V];
      vld<V>(a.w + i, w);
      vld<V>(a.p + n, p);
      vld<V>(a.Ap + n, ap);
      vld<V>(a.r + n, r);
      vst<V>(AP + head * ring + n, ap);
#pragma unroll
      for (int l = 0; l < V; ++l) {
        pap += w[l] * p[l] * ap[l];
        rp += w[l] * r[l] * p[l];
      }
    }
  }
  double v[2] = {(double)pap, (double)rp};
  if (grid_sum<2>(v, a.partials, a.counter)) {
    const double pAp = v[0], alpha = v[1] / pAp;
    st->pAp = pAp;
    if (!(pAp > 0.0) || !isfinite(alpha)) {
      st->done = 1;
      st->result = st->iter - 1;
      st->status = NEKB_ERR_BREAKDOWN;
      return;
    }
    st->alpha = alpha;
    st->fcg_pap[head] = pAp;
    st->fcg_head = (head + 1) % st->fcg_m;
    st->fcg_count = st->fcg_count < st->fcg_m ? st->fcg_count + 1 : st->fcg_m;
  }
}

// pAp from the operator's per-block sums of p . (A p)_local.  For a p that is
// continuous across element copies and zero on masked nodes, the
// invDegree-weighted sum of p . mask(gs(A_local p)) equals the plain sum of
// p . A_local p over all local nodes, so the operator kernel can form it in
// its epilogue and no pass over p and Ap is needed; alpha = rdotz / pAp.
__global__ void __launch_bounds__(1024) k_pap_partials(PcgState* st, const double* __restrict__ part,
                                                       const int* __restrict__ count)
{
  if (st->done) return;
  __shared__ double sh[32];
  const int n = *count;
  double v = 0.0;
  for (int b = threadIdx.x; b < n; b += blockDim.x) v += part[b];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double pAp = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) pAp += sh[w];
    const double alpha = st->rdotz1 / pAp;
    st->pAp = pAp;
    if (!(pAp > 0.0) || !isfinite(alpha)) {
      st->done = 1;
      st->result = st->iter - 1;
      st->status = NEKB_ERR_BREAKDOWN;
      return;
    }
    st->alpha = alpha;
  }
}

// pAp = sum w p Ap ; alpha = rdotz / pAp
template <typename T, int V = 1>
__global__ void __launch_bounds__(RT) k_pap(PcgArgs<T> a)
{
  PcgState* st = a.st;
  if (st->done) return;
  T acc = 0;
  const int64_t stride = (int64_t)gridDim.x * RT;
  const int64_t nv = a.Nloc / V;
  for (int f = 0; f < a.NF; ++f) {
    const int64_t fo = f * a.offset;
    for (int64_t iv = (int64_t)blockIdx.x * RT + threadIdx.x; iv < nv; iv += stride) {
      T w[V], p[V], ap[V];
      vld<V>(a.w + iv * V, w);
      vld<V>(a.p + iv * V + fo, p);
      vld<V>(a.Ap + iv * V + fo, ap);
#pragma unroll
      for (int l = 0; l < V; ++l) acc += w[l] * p[l] * ap[l];
    }
  }
  double v[1] = {(double)acc};
  if (grid_sum<1>(v, a.partials, a.counter)) {
    const double pAp = v[0];
    const double alpha = st->rdotz1 / pAp;
    st->pAp = pAp;
    if (!(pAp > 0.0) || !isfinite(alpha)) {
      st->done = 1;
      st->result = st->iter - 1;
      st->status = NEKB_ERR_BREAKDOWN;
      return;
    }
    st->alpha = alpha;
  }
}

}  // namespace

// out[0] = sum w u v over fields (weightedMultipleInnerProduct2, utils.okl:413);
// with TWO also out[1] = sum w u u (weightedInnerProductUpdate, utils.okl:687)
template <typename T, bool TWO>
__global__ void __launch_bounds__(RT) k_wdot(PcgArgs<T> a, const T* u, const T* v2)
{
  T acc = 0, acc2 = 0;
  const int64_t stride = (int64_t)gridDim.x * RT;
  for (int f = 0; f < a.NF; ++f) {
    const int64_t fo = f * a.offset;
    for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < a.Nloc; i += stride) {
      const T wu = a.w[i] * u[i + fo];
      acc += wu * v2[i + fo];
      if (TWO) acc2 += wu * u[i + fo];
    }
  }
  if (TWO) {
    double v[2] = {(double)acc, (double)acc2};
    if (grid_sum<2>(v, a.partials, a.counter)) {
      a.out[0] = v[0];
      a.out[1] = v[1];
    }
  } else {
    double v[1] = {(double)acc};
    if (grid_sum<1>(v, a.partials, a.counter)) *a.out = v[0];
  }
}

// launch of the weighted inner products on caller-provided scratch: partials
// (NV doubles per block), a zeroed counter, and out (NV doubles, device)
int launch_wdot(int64_t N, int NF, int64_t offset, const double* w, const double* u,
                const double* v, bool two, int64_t grid, double* partials, unsigned* counter,
                double* out, cudaStream_t s)
{
  PcgArgs<double> a{};
  a.Nloc = N;
  a.offset = offset;
  a.NF = NF;
  a.w = w;
  a.partials = partials;
  a.counter = counter;
  a.out = out;
  if (grid < 1 || grid > INT32_MAX) return fail(NEKB_ERR_INVALID, "weighted inner product: grid %lld", (long long)grid);
  if (two)
    k_wdot<double, true><<<(unsigned)grid, RT, 0, s>>>(a, u, v);
  else
    k_wdot<double, false><<<(unsigned)grid, RT, 0, s>>>(a, u, v);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

namespace {

// y = alpha x + beta y
template <typename T>
__global__ void k_axpby(int64_t N, T alpha, const T* x, T beta, T* y)
{
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    y[n] = alpha * x[n] + beta * y[n];
}

// r = b - Ax (FP64)
__global__ void k_residual(int64_t N, const double* b, const double* Ax, double* r)
{
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    r[n] = b[n] - Ax[n];
}

// r32 = float(s * r64)
__global__ void k_scale_down(int64_t N, double s, const double* r, float* r32)
{
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    r32[n] = (float)(s * r[n]);
}

// x64 += s * x32
__global__ void k_correct(int64_t N, double s, const float* x32, double* x)
{
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
    x[n] += s * (double)x32[n];
}

// mask list entries set to a value (updateJacobi's mapB==1 nodes, updateJacobi.okl:77-79)
__global__ void k_mask_set(int64_t Nm, const int32_t* ids, double v, double* q)
{
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < Nm; n += (int64_t)gridDim.x * blockDim.x)
    q[ids[n]] = v;
}

inline unsigned red_grid(int64_t n)
{
  int64_t b = (n + RT - 1) / RT;
  if (b < 1) b = 1;
  if (b > kMaxRedBlocks) b = kMaxRedBlocks;
  return (unsigned)b;
}

inline unsigned vec_grid(int64_t n)
{
  int64_t b = (n + RT - 1) / RT;
  if (b < 1) b = 1;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)b;
}

// the external (learned) preconditioner: z = M(r), launched on the stream;
// with m > 1 the iteration is FCG(m) on the ring buffers P, AP
struct ExtPrecond {
  nekb_bp* bp = nullptr;
  nekb_net* net = nullptr;
  const float* invDiag = nullptr;
  const float* w = nullptr;
  int m = 1;
  float* P = nullptr;
  float* AP = nullptr;
  // FP32 operator with the pAp sums fused into its epilogue (null: separate pass)
  double* axdot = nullptr;
  int* axdot_count = nullptr;
};

template <typename T, bool REFRESH>
int launch_fcg_dots(const PcgArgs<T>& a, const ExtPrecond* ext, cudaStream_t s)
{
  if constexpr (sizeof(T) == 4) {
    const int64_t ring = a.NF * a.offset;
    if (a.Nloc % 4 == 0 && a.offset % 4 == 0)
      k_fcg_dots<T, 4, REFRESH><<<red_grid(a.Nloc / 4), RT, 0, s>>>(a, ext->AP, ring);
    else
      k_fcg_dots<T, 1, REFRESH><<<red_grid(a.Nloc), RT, 0, s>>>(a, ext->AP, ring);
    NEKB_CUDA(cudaGetLastError());
    return NEKB_OK;
  } else {
    return fail(NEKB_ERR_UNSUPPORTED, "FCG(m) runs in FP32 only");
  }
}

// float4 access when the vectors allow it (FP32, lengths and offsets multiples of 4)
template <typename T>
inline int vec_width(const PcgArgs<T>& a)
{
  return (sizeof(T) == 4 && a.Nloc % 4 == 0 && a.offset % 4 == 0) ? 4 : 1;
}

template <typename T, int MODE, bool UPDATE, bool REFRESH, int V>
void launch_rz_v(const PcgArgs<T>& a, bool flex, cudaStream_t s)
{
  const unsigned rg = red_grid(a.Nloc / V);
  if (flex)
    k_update_rz<T, MODE, UPDATE, true, REFRESH, V><<<rg, RT, 0, s>>>(a);
  else
    k_update_rz<T, MODE, UPDATE, false, REFRESH, V><<<rg, RT, 0, s>>>(a);
}

// k_update_rz for the runtime (mode, flex) pair and vector width
template <typename T, bool UPDATE, bool REFRESH>
int launch_rz(const PcgArgs<T>& a, int mode, bool flex, cudaStream_t s)
{
  const bool v4 = vec_width(a) == 4;
  if constexpr (sizeof(T) == 4) {
    if (v4) {
      if (mode == PC_EXTERNAL) launch_rz_v<T, PC_EXTERNAL, UPDATE, REFRESH, 4>(a, flex, s);
      else if (mode == PC_JACOBI) launch_rz_v<T, PC_JACOBI, UPDATE, REFRESH, 4>(a, flex, s);
      else launch_rz_v<T, PC_COPY, UPDATE, REFRESH, 4>(a, flex, s);
      NEKB_CUDA(cudaGetLastError());
      return NEKB_OK;
    }
  }
  if (mode == PC_EXTERNAL) launch_rz_v<T, PC_EXTERNAL, UPDATE, REFRESH, 1>(a, flex, s);
  else if (mode == PC_JACOBI) launch_rz_v<T, PC_JACOBI, UPDATE, REFRESH, 1>(a, flex, s);
  else launch_rz_v<T, PC_COPY, UPDATE, REFRESH, 1>(a, flex, s);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

// one FCG(m) iteration with the external preconditioner (FP32)
template <typename T>
int launch_fcg_iteration(const OpView& op, PcgArgs<T> a, const ExtPrecond* ext, cudaStream_t s)
{
  if constexpr (sizeof(T) == 4) {
    const int64_t Nall = a.NF * a.offset;
    const bool v4 = vec_width(a) == 4;
    if (v4) {
      k_fcg_pupdate<T, 4><<<vec_grid(Nall / 4), RT, 0, s>>>(a, ext->P, Nall);
    } else {
      k_fcg_pupdate<T, 1><<<vec_grid(Nall), RT, 0, s>>>(a, ext->P, Nall);
    }
    NEKB_CUDA(cudaGetLastError());
    NEKB_TRY(apply_op(op, a.p, a.Ap, &a.st->done, s));
    if (v4) {
      k_fcg_pap<T, 4><<<red_grid(a.Nloc / 4), RT, 0, s>>>(a, ext->AP, Nall);
    } else {
      k_fcg_pap<T, 1><<<red_grid(a.Nloc), RT, 0, s>>>(a, ext->AP, Nall);
    }
    NEKB_CUDA(cudaGetLastError());
    if (net_takes_update(ext->net)) {  // x += alpha p, r -= alpha Ap inside the network kernel
      const NetUpdate up{&a.st->alpha, a.Ap, a.p, a.x};
      NEKB_TRY(net_precondition_update(ext->bp, ext->net, up, a.r, a.z, ext->invDiag, ext->w, &a.st->done, s));
    } else {
      k_update<T><<<vec_grid(Nall), RT, 0, s>>>(a);
      NEKB_CUDA(cudaGetLastError());
      NEKB_TRY(net_precondition(ext->bp, ext->net, a.r, a.z, ext->invDiag, ext->w, &a.st->done, s));
    }
    return launch_fcg_dots<T, false>(a, ext, s);
  } else {
    return fail(NEKB_ERR_UNSUPPORTED, "FCG(m) runs in FP32 only");
  }
}

template <typename T>
int launch_iteration(const OpView& op, PcgArgs<T> a, int mode, bool flex, const ExtPrecond* ext,
                     cudaStream_t s)
{
  if (mode == PC_EXTERNAL && ext && ext->m > 1) return launch_fcg_iteration<T>(op, a, ext, s);
  const int64_t Nall = a.NF * a.offset;
  const int V = vec_width(a);
  const unsigned vg = vec_grid(Nall / V), rg = red_grid(a.Nloc / V);
  if constexpr (sizeof(T) == 4) {
    if (V == 4) {
      if (mode == PC_COPY)
        k_pupdate<T, PC_COPY, 4><<<vg, RT, 0, s>>>(a);
      else
        k_pupdate<T, PC_JACOBI, 4><<<vg, RT, 0, s>>>(a);
    }
  }
  if (V == 1) {
    if (mode == PC_COPY)
      k_pupdate<T, PC_COPY, 1><<<vg, RT, 0, s>>>(a);
    else
      k_pupdate<T, PC_JACOBI, 1><<<vg, RT, 0, s>>>(a);
  }
  NEKB_CUDA(cudaGetLastError());
  if (sizeof(T) == 4 && ext && ext->axdot) {
    // FP32 operator: pAp from the operator kernel's own partial sums
    NEKB_TRY(apply_op(op, a.p, a.Ap, &a.st->done, s, ext->axdot, ext->axdot_count));
    k_pap_partials<<<1, 1024, 0, s>>>(a.st, ext->axdot, ext->axdot_count);
  } else {
    NEKB_TRY(apply_op(op, a.p, a.Ap, &a.st->done, s));
    if constexpr (sizeof(T) == 4) {
      if (V == 4) k_pap<T, 4><<<rg, RT, 0, s>>>(a);
    }
    if (V == 1) k_pap<T, 1><<<rg, RT, 0, s>>>(a);
  }
  NEKB_CUDA(cudaGetLastError());
  if (mode == PC_EXTERNAL) {
    if constexpr (sizeof(T) == 4) {
      if (net_takes_update(ext->net)) {  // x += alpha p, r -= alpha Ap inside the network kernel
        const NetUpdate up{&a.st->alpha, a.Ap, a.p, a.x};
        NEKB_TRY(net_precondition_update(ext->bp, ext->net, up, a.r, a.z, ext->invDiag, ext->w, &a.st->done, s));
      } else {
        k_update<T><<<vec_grid(Nall), RT, 0, s>>>(a);
        NEKB_CUDA(cudaGetLastError());
        NEKB_TRY(net_precondition(ext->bp, ext->net, a.r, a.z, ext->invDiag, ext->w, &a.st->done, s));
      }
    } else {
      return fail(NEKB_ERR_UNSUPPORTED, "learned preconditioner runs in FP32 only");
    }
    return launch_rz<T, false, false>(a, mode, flex, s);
  }
  return launch_rz<T, true, false>(a, mode, flex, s);
}

template <typename T>
int launch_first_rz(PcgArgs<T> a, int mode, bool flex, const ExtPrecond* ext, cudaStream_t s)
{
  if (mode == PC_EXTERNAL) {
    if constexpr (sizeof(T) == 4) {
      NEKB_TRY(net_precondition(ext->bp, ext->net, a.r, a.z, ext->invDiag, ext->w, &a.st->done, s));
    }
    if (ext->m > 1) return launch_fcg_dots<T, false>(a, ext, s);
  }
  return launch_rz<T, false, false>(a, mode, flex, s);
}

template <typename T>
int wdot(nekb_bp* bp, const T* w, const T* u, const T* v, int NF, double* result)
{
  PcgArgs<T> a{};
  a.Nloc = bp->Nlocal;
  a.offset = bp->offset;
  a.NF = NF;
  a.w = w;
  a.partials = bp->partials.as<double>();
  a.counter = bp->counter.as<unsigned>() + 4;
  a.out = bp->partials.as<double>() + 3 * 4096;
  k_wdot<T, false><<<red_grid(a.Nloc), RT, 0, bp->stream>>>(a, u, v);
  NEKB_CUDA(cudaGetLastError());
  NEKB_CUDA(cudaMemcpyAsync(result, a.out, sizeof(double), cudaMemcpyDeviceToHost, bp->stream));
  NEKB_CUDA(cudaStreamSynchronize(bp->stream));
  return NEKB_OK;
}

// z = M r and the (r, z) sums again after the residual was replaced; the
// iteration count and the search direction stay
template <typename T>
int launch_refresh_rz(PcgArgs<T> a, int mode, bool flex, const ExtPrecond* ext, cudaStream_t s)
{
  if (mode == PC_EXTERNAL) {
    if constexpr (sizeof(T) == 4) {
      NEKB_TRY(net_precondition(ext->bp, ext->net, a.r, a.z, ext->invDiag, ext->w, &a.st->done, s));
    }
    if (ext->m > 1) return launch_fcg_dots<T, true>(a, ext, s);
  }
  return launch_rz<T, false, true>(a, mode, flex, s);
}

// called after every chunk with the state in bp->h_state; sets *finish to end
// the iteration (without a hook the iteration ends when the state says done)
template <typename T>
using ChunkHook = std::function<int(PcgArgs<T>& a, bool* finish)>;

// PCG on (r, x) with operator op.  Workspace p, z, Ap, Ax of Nfields*offset.
template <typename T>
int pcg_core(nekb_bp* bp, const OpView& op, T* r, T* x, const T* w, const T* invDiag, T* p, T* z,
             T* Ap, T* Ax, int mode, bool flex, bool x_is_zero, double tol, int maxit,
             bool fixed, int chunk, bool use_graph, const ExtPrecond* ext, int* iters, int* status,
             double* rdotr0, double* rdotr, const ChunkHook<T>* hook = nullptr)
{
  cudaStream_t s = bp->stream;
  const int NF = op.Nfields;
  const int64_t Nall = NF * bp->offset;
  if (!x_is_zero) {
    NEKB_TRY(apply_op(op, x, Ax, nullptr, s));
    k_axpby<T><<<vec_grid(Nall), RT, 0, s>>>(Nall, T(-1), Ax, T(1), r);
    NEKB_CUDA(cudaGetLastError());
  }
  NEKB_CUDA(cudaMemsetAsync(p, 0, sizeof(T) * Nall, s));
  NEKB_CUDA(cudaMemsetAsync(Ap, 0, sizeof(T) * Nall, s));

  PcgState h{};
  h.rdotz1 = 1.0;
  h.rdotz2 = 0.0;
  h.alpha = 0.0;
  h.beta = 0.0;
  h.tol2 = tol * tol;
  h.maxit = maxit;
  h.flexible = flex ? 1 : 0;
  h.fixed = fixed ? 1 : 0;
  h.fcg_m = (mode == PC_EXTERNAL && ext && ext->m > 1) ? ext->m : 1;
  h.fcg_count = 0;
  h.fcg_head = 0;
  PcgState* st = bp->state.as<PcgState>();
  *bp->h_state = h;
  NEKB_CUDA(cudaMemcpyAsync(st, bp->h_state, sizeof(PcgState), cudaMemcpyHostToDevice, s));

  PcgArgs<T> a{};
  a.Nloc = bp->Nlocal;
  a.offset = bp->offset;
  a.NF = NF;
  a.w = w;
  a.invDiag = invDiag;
  a.r = r;
  a.x = x;
  a.p = p;
  a.z = z;
  a.Ap = Ap;
  a.st = st;
  a.partials = bp->partials.as<double>();
  a.counter = bp->counter.as<unsigned>();
  NEKB_TRY(launch_first_rz<T>(a, mode, flex, ext, s));

  if (chunk < 1) chunk = 1;
  cudaGraphExec_t gexec = nullptr;
  if (use_graph) {
    const NetSignature ns = net_signature(ext ? ext->net : nullptr);
    auto key = std::make_tuple(op.precision * 64 + mode * 4 + (flex ? 2 : 0) + (int)(sizeof(T) == 8),
                               chunk, op.flags, (const void*)op.lambda, (const void*)r, (const void*)x,
                               (int)(ext && ext->net ? 1 + ext->m : 0), ns.net, ns.weights, ns.shape_mode);
    auto it = bp->graphs.find(key);
    if (it != bp->graphs.end()) {
      gexec = it->second;
    } else {
      // one plain launch of the operator first (p = 0, so Ap stays 0): kernel
      // attributes are then set outside the capture
      NEKB_TRY(apply_op(op, p, Ap, &st->done, s));
      cudaGraph_t g = nullptr;
      NEKB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      int st_cap = NEKB_OK;
      for (int c = 0; c < chunk && st_cap == NEKB_OK; ++c)
        st_cap = launch_iteration<T>(op, a, mode, flex, ext, s);
      cudaError_t ce = cudaStreamEndCapture(s, &g);
      if (st_cap != NEKB_OK) {
        if (g) cudaGraphDestroy(g);
        return st_cap;
      }
      if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
      ce = cudaGraphInstantiate(&gexec, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) return cuda_fail(ce, "cudaGraphInstantiate", __FILE__, __LINE__);
      bp->graphs[key] = gexec;
    }
  }

  // a hook may resume a finished state (residual replacement): allow for that
  const int max_chunks = (maxit + 1 + chunk - 1) / chunk + 1 + (hook ? 256 : 0);
  for (int c = 0; c < max_chunks; ++c) {
    if (gexec) {
      NEKB_CUDA(cudaGraphLaunch(gexec, s));
    } else {
      for (int k = 0; k < chunk; ++k) NEKB_TRY(launch_iteration<T>(op, a, mode, flex, ext, s));
    }
    NEKB_CUDA(cudaMemcpyAsync(bp->h_state, st, sizeof(PcgState), cudaMemcpyDeviceToHost, s));
    NEKB_CUDA(cudaStreamSynchronize(s));
    if (hook) {
      bool finish = false;
      NEKB_TRY((*hook)(a, &finish));
      if (finish) break;
    } else if (bp->h_state->done) {
      break;
    }
  }
  const PcgState& hs = *bp->h_state;
  if (hook) {  // the hook decided; completed iterations = rz evaluations - 1
    *iters = hs.iter - 1;
    *status = hs.status;
    *rdotr0 = hs.rdotr0;
    *rdotr = hs.rdotr;
    return NEKB_OK;
  }
  if (!hs.done) return fail(NEKB_ERR_CUDA, "PCG: iteration state did not terminate");
  *iters = hs.result;
  *status = hs.status;
  *rdotr0 = hs.rdotr0;
  *rdotr = hs.rdotr;
  return NEKB_OK;
}

// Homogeneous Dirichlet nodes carry no unknown: zero them in the right-hand
// side and the initial guess so the masked operator stays symmetric.
int mask_rhs_guess(nekb_bp* bp, double* r, double* x)
{
  NEKB_TRY(launch_mask(bp->Nmasked, bp->mask.as<int32_t>(), bp->Nfields, bp->offset, r,
                       NEKB_DOUBLE, nullptr, bp->stream));
  NEKB_TRY(launch_mask(bp->Nmasked, bp->mask.as<int32_t>(), bp->Nfields, bp->offset, x,
                       NEKB_DOUBLE, nullptr, bp->stream));
  return NEKB_OK;
}

int ensure_jacobi64(nekb_bp* bp, int bk, const double* lambda)
{
  cudaStream_t s = bp->stream;
  double* d = bp->invDiag.as<double>();
  NEKB_TRY(launch_update_jacobi(bp->Nq, bp->E, bp->offset, nullptr, bp->ggeo.as<double>(),
                                bp->D.as<double>(), lambda, bk, d, s));
  if (bp->Nmasked > 0) {
    k_mask_set<<<vec_grid(bp->Nmasked), RT, 0, s>>>(bp->Nmasked, bp->mask.as<int32_t>(), 1.0, d);
    NEKB_CUDA(cudaGetLastError());
  }
  NEKB_TRY(launch_gs_add(bp->ogs, 1, bp->offset, d, NEKB_DOUBLE, nullptr, s));
  NEKB_TRY(launch_vec_inv(d, bp->offset, s));
  return NEKB_OK;
}

}  // namespace

OpView make_op(nekb_bp* bp, int bk, int precision, const void* lambda)
{
  OpView op;
  op.Nq = bp->Nq;
  op.flags = (bk ? NEKB_AX_BK : 0) | (bp->Nfields == 3 ? NEKB_AX_N3 : 0);
  op.precision = precision;
  op.Nfields = bp->Nfields;
  op.E = bp->E;
  op.offset = bp->offset;
  op.lambda = lambda;
  op.ogs = bp->ogs;
  op.mask = bp->mask.as<int32_t>();
  op.Nmasked = bp->Nmasked;
  for (int i = 0; i < bp->Nq; ++i) {
    op.r1d[i] = (float)bp->r1d[i];
    op.w1d[i] = (float)bp->w1d[i];
  }
  switch (precision) {
    case NEKB_FP64: op.ggeo = bp->ggeo.p; op.D = bp->D.p; break;
    case NEKB_FP32: op.ggeo = bp->ggeo_f.p; op.D = bp->Df.p; break;
    case NEKB_BF16: op.ggeo = bp->ggeo_bf.p; op.D = bp->Df.p; break;
    case NEKB_FP32_TRILINEAR: op.ggeo = bp->tri.p; op.D = bp->Df.p; break;
    case NEKB_FP64_SPLIT: op.ggeo = bp->ggeo.p; op.D = bp->D.p; break;
  }
  return op;
}

// lower-precision copies of geometry, lambda, weights and the Jacobi diagonal
int prepare_inner(nekb_bp* bp, int precision, int bk, const double* lambda, bool jacobi)
{
  cudaStream_t s = bp->stream;
  const int64_t Nl = bp->Nlocal;
  const int64_t Nall = bp->Nfields * bp->offset;
  for (DeviceBuf* w : {&bp->r32, &bp->x32, &bp->p32, &bp->z32, &bp->Ap32})
    NEKB_TRY(w->ensure(sizeof(float) * Nall));
  if (bp->invdeg_f.p == nullptr) {
    NEKB_TRY(bp->invdeg_f.ensure(sizeof(float) * Nl));
    NEKB_TRY(launch_convert_d2f(bp->ogs->d_invDegree, bp->invdeg_f.as<float>(), Nl, s));
  }
  if (precision == NEKB_FP32 && bp->ggeo_f.p == nullptr) {
    NEKB_TRY(bp->ggeo_f.ensure(sizeof(float) * 7 * Nl));
    NEKB_TRY(launch_convert_d2f(bp->ggeo.as<double>(), bp->ggeo_f.as<float>(), 7 * Nl, s));
  }
  if (precision == NEKB_BF16 && bp->ggeo_bf.p == nullptr) {
    NEKB_TRY(bp->ggeo_bf.ensure(sizeof(__nv_bfloat16) * 7 * Nl));
    NEKB_TRY(launch_convert_d2bf(bp->ggeo.as<double>(), bp->ggeo_bf.as<__nv_bfloat16>(), 7 * Nl, s));
  }
  if (!bk) {
    if (lambda == nullptr) return fail(NEKB_ERR_INVALID, "PCG: lambda is NULL for a Helmholtz solve");
    if (precision == NEKB_BF16) {
      NEKB_TRY(bp->lam32.ensure(sizeof(__nv_bfloat16) * 2 * Nl));
      NEKB_TRY(launch_convert_d2bf(lambda, bp->lam32.as<__nv_bfloat16>(), 2 * Nl, s));
    } else {
      NEKB_TRY(bp->lam32.ensure(sizeof(float) * 2 * Nl));
      NEKB_TRY(launch_convert_d2f(lambda, bp->lam32.as<float>(), 2 * Nl, s));
    }
  }
  if (jacobi) {
    NEKB_TRY(ensure_jacobi64(bp, bk, lambda));
    NEKB_TRY(bp->invDiag32.ensure(sizeof(float) * Nl));
    NEKB_TRY(launch_convert_d2f(bp->invDiag.as<double>(), bp->invDiag32.as<float>(), Nl, s));
  }
  return NEKB_OK;
}

int solve_fp64(nekb_bp* bp, const double* lambda, double* r, double* x, double tol, int maxit,
               const nekb_pcg_opts& o, nekb_pcg_stats* stats)
{
  cudaStream_t s = bp->stream;
  const int64_t Nall = bp->Nfields * bp->offset;
  if (!o.bk && lambda == nullptr) return fail(NEKB_ERR_INVALID, "PCG: lambda is NULL for a Helmholtz solve");
  if (o.precond == NEKB_PRECOND_LEARNED) return fail(NEKB_ERR_UNSUPPORTED, "learned preconditioner needs the mixed solver");
  // the Krylov operator: native FP64, or double-float on the FP32 pipes
  // (NEKB_SOLVER_FP64_SPLIT); the final true residual always uses native FP64
  const OpView op64 = make_op(bp, o.bk, NEKB_FP64, lambda);
  const OpView op = o.solver == NEKB_SOLVER_FP64_SPLIT ? make_op(bp, o.bk, NEKB_FP64_SPLIT, lambda) : op64;
  NEKB_TRY(bp->b.ensure(sizeof(double) * Nall));
  NEKB_TRY(bp->rr.ensure(sizeof(double) * Nall));
  NEKB_TRY(mask_rhs_guess(bp, r, x));
  NEKB_CUDA(cudaMemcpyAsync(bp->b.p, r, sizeof(double) * Nall, cudaMemcpyDeviceToDevice, s));
  const int mode = o.precond == NEKB_PRECOND_JACOBI ? PC_JACOBI : PC_COPY;
  if (mode == PC_JACOBI) NEKB_TRY(ensure_jacobi64(bp, o.bk, lambda));
  int iters = 0, status = 0;
  double rdotr0 = 0, rdotr = 0;
  NEKB_TRY(pcg_core<double>(bp, op, r, x, bp->ogs->d_invDegree, bp->invDiag.as<double>(),
                            bp->p.as<double>(), bp->z.as<double>(), bp->Ap.as<double>(),
                            bp->Ax.as<double>(), mode, o.flexible != 0, false, tol, maxit,
                            o.fixed_iterations != 0, o.check_every, o.use_graph != 0, nullptr,
                            &iters, &status, &rdotr0, &rdotr));
  // true FP64 residual |b - A x|_w / |b - A x0|_w
  NEKB_TRY(apply_op(op64, x, bp->Ax.p, nullptr, s));
  k_residual<<<vec_grid(Nall), RT, 0, s>>>(Nall, bp->b.as<double>(), bp->Ax.as<double>(), bp->rr.as<double>());
  NEKB_CUDA(cudaGetLastError());
  double tr = 0;
  NEKB_TRY(wdot<double>(bp, bp->ogs->d_invDegree, bp->rr.as<double>(), bp->rr.as<double>(), bp->Nfields, &tr));
  stats->iterations = iters;
  stats->outer_iterations = 1;
  stats->status = status;
  stats->rdotr0 = rdotr0;
  stats->rdotr = rdotr;
  stats->true_rel_res = rdotr0 > 0 ? std::sqrt(tr / rdotr0) : std::sqrt(tr);
  return NEKB_OK;
}

// Mixed precision: the Krylov iteration runs in FP32 (operator in FP32, BF16
// storage or FP32 with trilinear geometry) and the solution and true residual
// are kept in FP64; the FP32 residual is replaced by the FP64 one every time it
// has dropped by inner_tol (default 1e-2), so the reported residual is always
// the true FP64 |b - A x|_w and no Krylov information is lost to restarts.
int solve_mixed(nekb_bp* bp, const double* lambda, double* r, double* x, double tol, int maxit,
                const nekb_pcg_opts& o, nekb_pcg_stats* stats)
{
  cudaStream_t s = bp->stream;
  const int64_t Nall = bp->Nfields * bp->offset;
  const int prec = o.inner_precision;
  if (prec != NEKB_FP32 && prec != NEKB_BF16 && prec != NEKB_FP32_TRILINEAR)
    return fail(NEKB_ERR_INVALID, "mixed solver: inner precision %d", prec);
  if (prec == NEKB_FP32_TRILINEAR && bp->tri.p == nullptr)
    return fail(NEKB_ERR_UNSUPPORTED, "mixed solver: trilinear geometry needs the element vertices");
  if (!o.bk && lambda == nullptr) return fail(NEKB_ERR_INVALID, "PCG: lambda is NULL for a Helmholtz solve");
  const bool learned = o.precond == NEKB_PRECOND_LEARNED;
  const bool jacobi = o.precond == NEKB_PRECOND_JACOBI || learned;
  if (learned && o.net == nullptr) return fail(NEKB_ERR_INVALID, "learned preconditioner: net is NULL");
  NEKB_TRY(prepare_inner(bp, prec, o.bk, lambda, jacobi));
  OpView op64 = make_op(bp, o.bk, NEKB_FP64, lambda);
  OpView op32 = make_op(bp, o.bk, prec, o.bk ? nullptr : bp->lam32.p);
  NEKB_TRY(bp->b.ensure(sizeof(double) * Nall));
  NEKB_TRY(bp->rr.ensure(sizeof(double) * Nall));
  double* b = bp->b.as<double>();
  NEKB_TRY(mask_rhs_guess(bp, r, x));
  NEKB_CUDA(cudaMemcpyAsync(b, r, sizeof(double) * Nall, cudaMemcpyDeviceToDevice, s));
  // r = b - A x
  NEKB_TRY(apply_op(op64, x, bp->Ax.p, nullptr, s));
  k_residual<<<vec_grid(Nall), RT, 0, s>>>(Nall, b, bp->Ax.as<double>(), r);
  NEKB_CUDA(cudaGetLastError());
  double rdotr0 = 0;
  NEKB_TRY(wdot<double>(bp, bp->ogs->d_invDegree, r, r, bp->Nfields, &rdotr0));
  const double TOL = std::fmax(tol * tol * rdotr0, tol * tol);
  double rdotr = rdotr0;
  int total = 0, outer = 0, status = NEKB_OK;
  const int max_outer = o.max_outer > 0 ? o.max_outer : 20;
  // residual reduction (in norm) between two replacements of the FP32
  // recursive residual by the true FP64 one
  const double delta = o.inner_tol > 0 ? o.inner_tol : 1e-2;
  ExtPrecond ext;
  ext.bp = bp;
  ext.net = (nekb_net*)o.net;
  ext.invDiag = bp->invDiag32.as<float>();
  ext.w = bp->invdeg_f.as<float>();
  {
    // one partial per operator block: at most one block per element
    NEKB_TRY(bp->axdot.ensure(sizeof(double) * (bp->E + 8)));
    ext.axdot = bp->axdot.as<double>() + 8;
    ext.axdot_count = reinterpret_cast<int*>(bp->axdot.as<double>());
  }
  if (learned) {
    ext.m = o.fcg_window > 0 ? o.fcg_window : 5;
    if (ext.m > kFcgMax) return fail(NEKB_ERR_INVALID, "fcg_window %d > %d", o.fcg_window, kFcgMax);
    if (ext.m > 1) {
      // sized for the longest window once, so captured graphs keep valid pointers
      NEKB_TRY(bp->fcgP.ensure(sizeof(float) * kFcgMax * Nall));
      NEKB_TRY(bp->fcgAP.ensure(sizeof(float) * kFcgMax * Nall));
      ext.P = bp->fcgP.as<float>();
      ext.AP = bp->fcgAP.as<float>();
    }
  }
  const int mode = learned ? PC_EXTERNAL : (jacobi ? PC_JACOBI : PC_COPY);
  const bool flex = learned || o.flexible != 0;
  if (rdotr > TOL) {
    // One FP32 Krylov run on the scaled problem (|r0| = 1).  Whenever its
    // recursive residual has dropped by delta since the last replacement (or
    // it believes it converged), the FP32 correction is folded into the FP64
    // x, the true residual r = b - A64 x is formed in FP64, and it replaces
    // the FP32 residual; the search direction is kept (reliable updates).
    const double s0 = 1.0 / std::sqrt(rdotr0);
    float* r32 = bp->r32.as<float>();
    float* x32 = bp->x32.as<float>();
    k_scale_down<<<vec_grid(Nall), RT, 0, s>>>(Nall, s0, r, r32);
    NEKB_CUDA(cudaGetLastError());
    NEKB_CUDA(cudaMemsetAsync(x32, 0, sizeof(float) * Nall, s));
    double rr_last = 1.0;  // scaled |r|^2 at the last replacement
    const double TOL32 = TOL * s0 * s0;
    auto fold = [&]() -> int {  // x += x32/s0 ; x32 = 0 ; r = b - A x ; rdotr
      k_correct<<<vec_grid(Nall), RT, 0, s>>>(Nall, 1.0 / s0, x32, x);
      NEKB_CUDA(cudaGetLastError());
      NEKB_CUDA(cudaMemsetAsync(x32, 0, sizeof(float) * Nall, s));
      NEKB_TRY(apply_op(op64, x, bp->Ax.p, nullptr, s));
      k_residual<<<vec_grid(Nall), RT, 0, s>>>(Nall, b, bp->Ax.as<double>(), r);
      NEKB_CUDA(cudaGetLastError());
      NEKB_TRY(wdot<double>(bp, bp->ogs->d_invDegree, r, r, bp->Nfields, &rdotr));
      outer++;
      return NEKB_OK;
    };
    // BF16 storage perturbs the operator by ~1e-3: Krylov directions built with
    // it do not stay conjugate for the true operator, so there each replacement
    // restarts the iteration (iterative refinement); FP32 operators keep p.
    const bool restart = (prec == NEKB_BF16);
    int done_before = 0;  // iterations of finished restarted segments
    ChunkHook<float> hook = [&](PcgArgs<float>& a, bool* finish) -> int {
      PcgState& hs = *bp->h_state;
      if (o.fixed_iterations) {  // exactly maxit iterations, then one fold
        if (hs.done) {
          NEKB_TRY(fold());
          *finish = true;
        }
        return NEKB_OK;
      }
      const bool stop = hs.done && hs.status != NEKB_OK;  // breakdown or iteration limit
      if (!(hs.done || hs.rdotr < delta * delta * rr_last)) return NEKB_OK;
      NEKB_TRY(fold());
      if (rdotr <= TOL || stop || outer >= max_outer) {
        if (hs.status == NEKB_ERR_BREAKDOWN) status = NEKB_ERR_BREAKDOWN;
        *finish = true;
        return NEKB_OK;
      }
      // replace the FP32 residual and resume the same iteration
      k_scale_down<<<vec_grid(Nall), RT, 0, s>>>(Nall, s0, r, r32);
      NEKB_CUDA(cudaGetLastError());
      rr_last = rdotr * s0 * s0;
      hs.done = 0;
      hs.status = NEKB_OK;
      hs.TOL = TOL32;
      if (restart) {
        // a fresh iteration: p = 0, rdotz1 = 1, alpha = beta = 0, counter reset
        // (iterations so far are kept in done_before; the budget shrinks)
        const int it_seg = hs.iter - 1;
        done_before += it_seg > 0 ? it_seg : 0;
        if (done_before >= maxit) {
          status = NEKB_ERR_NOT_CONVERGED;
          *finish = true;
          return NEKB_OK;
        }
        hs.iter = 0;
        hs.maxit = maxit - done_before;
        hs.rdotz1 = 1.0;
        hs.rdotz2 = 0.0;
        hs.alpha = 0.0;
        hs.beta = 0.0;
        hs.fcg_count = 0;
        hs.fcg_head = 0;
        NEKB_CUDA(cudaMemsetAsync(a.p, 0, sizeof(float) * Nall, s));
        NEKB_CUDA(cudaMemsetAsync(a.Ap, 0, sizeof(float) * Nall, s));
        NEKB_CUDA(cudaMemcpyAsync(a.st, &hs, sizeof(PcgState), cudaMemcpyHostToDevice, s));
        return launch_first_rz<float>(a, mode, flex, &ext, s);
      }
      NEKB_CUDA(cudaMemcpyAsync(a.st, &hs, sizeof(PcgState), cudaMemcpyHostToDevice, s));
      NEKB_TRY(launch_refresh_rz<float>(a, mode, flex, &ext, s));
      return NEKB_OK;
    };
    int it = 0, st = 0;
    double a0 = 0, a1 = 0;
    NEKB_TRY(pcg_core<float>(bp, op32, r32, x32, bp->invdeg_f.as<float>(),
                             bp->invDiag32.as<float>(), bp->p32.as<float>(), bp->z32.as<float>(),
                             bp->Ap32.as<float>(), bp->Ap32.as<float>(), mode, flex, true,
                             std::sqrt(TOL32), maxit, o.fixed_iterations != 0, o.check_every,
                             o.use_graph != 0,
                             &ext, &it, &st, &a0, &a1, &hook));
    total = it + done_before;
    if (learned) NEKB_TRY(net_tc_copy_timeout());
    if (st == NEKB_ERR_BREAKDOWN) status = st;
  }
  if (rdotr > TOL && status == NEKB_OK && !o.fixed_iterations) status = NEKB_ERR_NOT_CONVERGED;
  stats->iterations = total;
  stats->outer_iterations = outer;
  stats->status = status;
  stats->rdotr0 = rdotr0;
  stats->rdotr = rdotr;
  stats->true_rel_res = rdotr0 > 0 ? std::sqrt(rdotr / rdotr0) : std::sqrt(rdotr);
  return NEKB_OK;
}

int bp_pcg(nekb_bp* bp, const double* lambda, double* r, double* x, double tol, int maxit,
           const nekb_pcg_opts* opts, nekb_pcg_stats* stats)
{
  nekb_pcg_opts o;
  if (opts) {
    o = *opts;
  } else {
    std::memset(&o, 0, sizeof(o));
    o.precond = NEKB_PRECOND_JACOBI;
    o.check_every = 16;
    o.use_graph = 1;
  }
  if (!bp || !r || !x || !stats) return fail(NEKB_ERR_INVALID, "PCG: NULL argument");
  if (maxit < 0 || !(tol >= 0)) return fail(NEKB_ERR_INVALID, "PCG: maxit=%d tol=%g", maxit, tol);
  if (o.check_every <= 0) o.check_every = 16;
  if (o.solver != NEKB_SOLVER_FP64 && o.solver != NEKB_SOLVER_MIXED && o.solver != NEKB_SOLVER_FP64_SPLIT)
    return fail(NEKB_ERR_INVALID, "PCG: unknown solver %d", o.solver);
  cudaEvent_t e0, e1;
  NEKB_CUDA(cudaEventCreate(&e0));
  NEKB_CUDA(cudaEventCreate(&e1));
  NEKB_CUDA(cudaEventRecord(e0, bp->stream));
  int st = NEKB_OK;
  if (o.zero_mean) st = bp_zero_mean(bp, r);  // solve(), nekBone/main.cpp:24-25
  if (st == NEKB_OK) {
    if (o.solver == NEKB_SOLVER_MIXED)
      st = solve_mixed(bp, lambda, r, x, tol, maxit, o, stats);
    else
      st = solve_fp64(bp, lambda, r, x, tol, maxit, o, stats);
  }
  if (o.zero_mean && st == NEKB_OK) {
    const int zs = bp_zero_mean(bp, x);  // nekBone/main.cpp:30-31
    if (zs != NEKB_OK) st = zs;
  }
  cudaEventRecord(e1, bp->stream);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st == NEKB_OK) stats->elapsed_s = ms * 1e-3;
  return st;
}

namespace {

// sum kernel (utils.okl:212): per node the sum over fields, deterministic grid sum
__global__ void __launch_bounds__(RT) k_field_sum(int64_t N, int NF, int64_t offset,
                                                  const double* __restrict__ q, double* partials,
                                                  unsigned* counter, double* out)
{
  double acc = 0.0;
  const int64_t stride = (int64_t)gridDim.x * RT;
  for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < N; i += stride)
    for (int f = 0; f < NF; ++f) acc += q[i + f * offset];
  double v[1] = {acc};
  if (grid_sum<1>(v, partials, counter)) *out = v[0];
}

// addScalar (utils.okl:29) of minus the mean
__global__ void k_sub_mean(int64_t N, const double* __restrict__ sum, double count,
                           double* __restrict__ q)
{
  const double m = -(*sum / count);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x)
    q[i] += m;
}

}  // namespace

// BPZeroMean (solve.cpp:115-134)
int bp_zero_mean(nekb_bp* bp, double* q)
{
  if (!bp || !q) return fail(NEKB_ERR_INVALID, "zero mean: NULL argument");
  const int64_t N = bp->E * (int64_t)bp->Np, Nall = bp->Nfields * bp->offset;
  if (N == 0) return NEKB_OK;
  double* out = bp->partials.as<double>() + 3 * 4096 + 4;
  k_field_sum<<<red_grid(N), RT, 0, bp->stream>>>(N, bp->Nfields, bp->offset, q,
                                                  bp->partials.as<double>(),
                                                  bp->counter.as<unsigned>() + 12, out);
  NEKB_CUDA(cudaGetLastError());
  const unsigned g = (unsigned)std::min<int64_t>((Nall + 255) / 256, 152 * 16);
  k_sub_mean<<<g, 256, 0, bp->stream>>>(Nall, out, (double)(N * bp->Nfields), q);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int bp_wdot(nekb_bp* bp, const double* u, const double* v, double* out)
{
  return wdot<double>(bp, bp->ogs->d_invDegree, u, v, bp->Nfields, out);
}

// BPWeightedInnerProduct / BPWeightedInnerProduct2 on the problem's scratch;
// results returned to the host like the reference's host-side sums
int bp_weighted_inner_product(nekb_bp* bp, const double* w, const double* a, const double* b,
                              bool two, double* host_out)
{
  if (!bp || !w || !a || !b || !host_out) return fail(NEKB_ERR_INVALID, "weighted inner product: NULL argument");
  double* out = bp->partials.as<double>() + 3 * 4096;
  NEKB_TRY(launch_wdot(bp->Nlocal, bp->Nfields, bp->offset, w, a, b, two,
                       red_grid(bp->Nlocal), bp->partials.as<double>(),
                       bp->counter.as<unsigned>() + 8, out, bp->stream));
  NEKB_CUDA(cudaMemcpyAsync(host_out, out, sizeof(double) * (two ? 2 : 1), cudaMemcpyDeviceToHost, bp->stream));
  NEKB_CUDA(cudaStreamSynchronize(bp->stream));
  return NEKB_OK;
}

}  // namespace nekb
