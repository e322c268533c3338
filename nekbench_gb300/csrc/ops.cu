// Element-local operators other than axhelm's body, gather-scatter kernels and
// vector utilities.
#include "internal.h"

#include <algorithm>
#include <climits>
#include <cmath>

namespace nekb {

// ------------------------------------------------------------------ axhelm dispatch
#define NEKB_DECL_AX(P)                                                     \
  int launch_axhelm_##P##_nq2(int, const AxArgs&, cudaStream_t);            \
  int launch_axhelm_##P##_nq3(int, const AxArgs&, cudaStream_t);            \
  int launch_axhelm_##P##_nq4(int, const AxArgs&, cudaStream_t);            \
  int launch_axhelm_##P##_nq5(int, const AxArgs&, cudaStream_t);            \
  int launch_axhelm_##P##_nq6(int, const AxArgs&, cudaStream_t);            \
  int launch_axhelm_##P##_nq7(int, const AxArgs&, cudaStream_t);            \
  int launch_axhelm_##P##_nq8(int, const AxArgs&, cudaStream_t);            \
  int launch_axhelm_##P##_nq9(int, const AxArgs&, cudaStream_t);            \
  int launch_axhelm_##P##_nq10(int, const AxArgs&, cudaStream_t);           \
  int launch_axhelm_##P##_nq11(int, const AxArgs&, cudaStream_t);           \
  int launch_axhelm_##P##_nq12(int, const AxArgs&, cudaStream_t);
NEKB_DECL_AX(f64)
int launch_axhelm_f64_nq13(int, const AxArgs&, cudaStream_t);
int launch_axhelm_f64_nq14(int, const AxArgs&, cudaStream_t);
NEKB_DECL_AX(f32)
NEKB_DECL_AX(bf16)
NEKB_DECL_AX(tri)
NEKB_DECL_AX(x)

#define NEKB_SWITCH_AX(P)                                          \
  switch (Nq) {                                                    \
    case 2: return launch_axhelm_##P##_nq2(flags, a, s);           \
    case 3: return launch_axhelm_##P##_nq3(flags, a, s);           \
    case 4: return launch_axhelm_##P##_nq4(flags, a, s);           \
    case 5: return launch_axhelm_##P##_nq5(flags, a, s);           \
    case 6: return launch_axhelm_##P##_nq6(flags, a, s);           \
    case 7: return launch_axhelm_##P##_nq7(flags, a, s);           \
    case 8: return launch_axhelm_##P##_nq8(flags, a, s);           \
    case 9: return launch_axhelm_##P##_nq9(flags, a, s);           \
    case 10: return launch_axhelm_##P##_nq10(flags, a, s);         \
    case 11: return launch_axhelm_##P##_nq11(flags, a, s);         \
    case 12: return launch_axhelm_##P##_nq12(flags, a, s);         \
  }                                                                \
  break;

int launch_axhelm(int Nq, int flags, int precision, const AxArgs& a, cudaStream_t s)
{
  if (Nq < kMinNq || Nq > kMaxNq) return fail(NEKB_ERR_UNSUPPORTED, "axhelm: Nq=%d outside 2..%d", Nq, kMaxNq);
  if (flags & ~(NEKB_AX_BK | NEKB_AX_N3 | NEKB_AX_PARTIAL))
    return fail(NEKB_ERR_INVALID, "axhelm: unknown flag bits 0x%x", flags);
  if (precision != NEKB_FP64 && Nq > kMaxNqReduced)
    return fail(NEKB_ERR_UNSUPPORTED, "axhelm: Nq=%d is built for FP64 only (other precisions: Nq <= %d)",
                Nq, kMaxNqReduced);
  if (precision == NEKB_FP64 && Nq == 13) return launch_axhelm_f64_nq13(flags, a, s);
  if (precision == NEKB_FP64 && Nq == 14) return launch_axhelm_f64_nq14(flags, a, s);
  switch (precision) {
    case NEKB_FP64: NEKB_SWITCH_AX(f64)
    case NEKB_FP32: NEKB_SWITCH_AX(f32)
    case NEKB_BF16: NEKB_SWITCH_AX(bf16)
    case NEKB_FP32_TRILINEAR: NEKB_SWITCH_AX(tri)
    case NEKB_FP64_SPLIT: NEKB_SWITCH_AX(x)
    default: break;
  }
  return fail(NEKB_ERR_UNSUPPORTED, "axhelm: precision %d not supported", precision);
}

namespace {

inline unsigned grid_for(int64_t n, int threads, int64_t cap = 152 * 16)
{
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

// ------------------------------------------------------------------ Jacobi diagonal
// updateJacobi (nekBone/kernel/updateJacobi.okl:27-108): one thread per node,
// the reference's terms in its order.  Every product and sum is an explicitly
// rounded FP64 operation (no fused multiply-add), so the diagonal is bit for
// bit the CPU statement's; the kernel runs once per solve.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

template <bool bk>
__global__ void k_update_jacobi(int Nq, int64_t E, int64_t offset, const int32_t* __restrict__ mapB,
                                const double* __restrict__ ggeo, const double* __restrict__ D,
                                const double* __restrict__ lambda, double* __restrict__ diag)
{
  const int Np = Nq * Nq * Nq;
  const int64_t total = E * Np;
  for (int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = id / Np;
    const int n = (int)(id - e * Np);
    const int i = n % Nq, j = (n / Nq) % Nq, k = n / (Nq * Nq);
    double r_q = 1.0;
    if (!(mapB != nullptr && mapB[id] == 1)) {
      const double* g = ggeo + e * 7 * Np;
      const double* l0 = lambda + e * Np;
      const double lam0 = bk ? 1.0 : l0[n];
      const double lam1 = bk ? 0.0 : lambda[id + offset];
      const double Dii = D[i * Nq + i], Djj = D[j * Nq + j], Dkk = D[k * Nq + k];
      // 2 * G * lambda0 * Da * Db, left to right
      auto cross = [&](int slot, double Da, double Db) {
        return mul_rn(mul_rn(mul_rn(mul_rn(2.0, g[slot * Np + n]), lam0), Da), Db);
      };
      r_q = 0.0;
      r_q = add_rn(r_q, cross(2, Dii, Djj));
      r_q = add_rn(r_q, cross(3, Dii, Dkk));
      r_q = add_rn(r_q, cross(5, Djj, Dkk));
      for (int m = 0; m < Nq; ++m) {
        const int nr = m + Nq * (j + Nq * k), ns = i + Nq * (m + Nq * k), nt = i + Nq * (j + Nq * m);
        const double dmi = D[m * Nq + i], dmj = D[m * Nq + j], dmk = D[m * Nq + k];
        r_q = add_rn(r_q, mul_rn(mul_rn(mul_rn(g[1 * Np + nr], bk ? 1.0 : l0[nr]), dmi), dmi));
        r_q = add_rn(r_q, mul_rn(mul_rn(mul_rn(g[4 * Np + ns], bk ? 1.0 : l0[ns]), dmj), dmj));
        r_q = add_rn(r_q, mul_rn(mul_rn(mul_rn(g[6 * Np + nt], bk ? 1.0 : l0[nt]), dmk), dmk));
      }
      r_q = add_rn(r_q, mul_rn(g[n], lam1));
    }
    diag[id] = r_q;
  }
}

// ------------------------------------------------------------------ geometry
// Trilinear map of the 8 element vertices (vertex order of
// core/meshSetup.cpp:2363-2410) evaluated analytically at the GLL nodes:
// the same geometric factors meshGeometricFactorsHex3D (meshSetup.cpp:255-360)
// obtains by differentiating the nodal coordinates with D.
struct Nodes1D {
  double r[kMaxNq];
  double w[kMaxNq];
};

__device__ __forceinline__ void vertex_signs(int v, double& sr, double& ss, double& st)
{
  sr = (v == 1 || v == 2 || v == 5 || v == 6) ? 1.0 : -1.0;
  ss = (v == 2 || v == 3 || v == 6 || v == 7) ? 1.0 : -1.0;
  st = (v >= 4) ? 1.0 : -1.0;
}

__global__ void k_geometric_factors(int Nq, int64_t E, const double* __restrict__ EX,
                                    const double* __restrict__ EY, const double* __restrict__ EZ,
                                    Nodes1D nd, double* __restrict__ ggeo)
{
  const int Np = Nq * Nq * Nq;
  const int64_t total = E * Np;
  for (int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = id / Np;
    const int n = (int)(id - e * Np);
    const int i = n % Nq, j = (n / Nq) % Nq, k = n / (Nq * Nq);
    const double r = nd.r[i], s = nd.r[j], t = nd.r[k];
    double dx[3] = {0, 0, 0}, dy[3] = {0, 0, 0}, dz[3] = {0, 0, 0};
    for (int v = 0; v < 8; ++v) {
      double sr, ss, st;
      vertex_signs(v, sr, ss, st);
      const double fr = 0.125 * sr * (1.0 + ss * s) * (1.0 + st * t);
      const double fs = 0.125 * ss * (1.0 + sr * r) * (1.0 + st * t);
      const double ft = 0.125 * st * (1.0 + sr * r) * (1.0 + ss * s);
      const double X = EX[e * 8 + v], Y = EY[e * 8 + v], Z = EZ[e * 8 + v];
      dx[0] += fr * X; dx[1] += fs * X; dx[2] += ft * X;
      dy[0] += fr * Y; dy[1] += fs * Y; dy[2] += ft * Y;
      dz[0] += fr * Z; dz[1] += fs * Z; dz[2] += ft * Z;
    }
    const double xr = dx[0], xs = dx[1], xt = dx[2];
    const double yr = dy[0], ys = dy[1], yt = dy[2];
    const double zr = dz[0], zs = dz[1], zt = dz[2];
    const double J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
    const double rx = (ys * zt - zs * yt) / J, ry = -(xs * zt - zs * xt) / J, rz = (xs * yt - ys * xt) / J;
    const double sx = -(yr * zt - zr * yt) / J, sy = (xr * zt - zr * xt) / J, sz = -(xr * yt - yr * xt) / J;
    const double tx = (yr * zs - zr * ys) / J, ty = -(xr * zs - zr * xs) / J, tz = (xr * ys - yr * xs) / J;
    const double JW = J * nd.w[i] * nd.w[j] * nd.w[k];
    double* g = ggeo + e * 7 * Np + n;
    g[0 * Np] = JW;
    g[1 * Np] = JW * (rx * rx + ry * ry + rz * rz);
    g[2 * Np] = JW * (rx * sx + ry * sy + rz * sz);
    g[3 * Np] = JW * (rx * tx + ry * ty + rz * tz);
    g[4 * Np] = JW * (sx * sx + sy * sy + sz * sz);
    g[5 * Np] = JW * (sx * tx + sy * ty + sz * tz);
    g[6 * Np] = JW * (tx * tx + ty * ty + tz * tz);
  }
}

__global__ void k_physical_nodes(int Nq, int64_t E, const double* __restrict__ EX,
                                 const double* __restrict__ EY, const double* __restrict__ EZ,
                                 Nodes1D nd, double* x, double* y, double* z)
{
  const int Np = Nq * Nq * Nq;
  const int64_t total = E * Np;
  for (int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = id / Np;
    const int n = (int)(id - e * Np);
    const double r = nd.r[n % Nq], s = nd.r[(n / Nq) % Nq], t = nd.r[n / (Nq * Nq)];
    double X = 0, Y = 0, Z = 0;
    for (int v = 0; v < 8; ++v) {
      double sr, ss, st;
      vertex_signs(v, sr, ss, st);
      const double f = 0.125 * (1.0 + sr * r) * (1.0 + ss * s) * (1.0 + st * t);
      X += f * EX[e * 8 + v]; Y += f * EY[e * 8 + v]; Z += f * EZ[e * 8 + v];
    }
    x[id] = X; y[id] = Y; z[id] = Z;
  }
}

// coef[e*24 + comp*8 + a]: x(r,s,t) = sum_a coef_a * basis_a, basis {1,r,s,t,rs,rt,st,rst}
__global__ void k_trilinear_coeffs(int64_t E, const double* __restrict__ EX,
                                   const double* __restrict__ EY, const double* __restrict__ EZ,
                                   float* __restrict__ coef)
{
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double* V[3] = {EX + e * 8, EY + e * 8, EZ + e * 8};
    for (int comp = 0; comp < 3; ++comp) {
      double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int v = 0; v < 8; ++v) {
        double sr, ss, st;
        vertex_signs(v, sr, ss, st);
        const double X = 0.125 * V[comp][v];
        c[0] += X; c[1] += sr * X; c[2] += ss * X; c[3] += st * X;
        c[4] += sr * ss * X; c[5] += sr * st * X; c[6] += ss * st * X; c[7] += sr * ss * st * X;
      }
      for (int a = 0; a < 8; ++a) coef[e * 24 + comp * 8 + a] = (float)c[a];
    }
  }
}

// ------------------------------------------------------------------ gather-scatter
// gatherScatterMany_<type>Add (3rdParty/ogs/okl/gatherScatterMany.okl:58-85) over
// the groups that have more than one member (singleton groups are a no-op in
// the reference).  Each group's sum runs over its members in CSR order, so
// results are deterministic and equal to the CPU's.
//
// The kernel is bound by the latency of its dependent loads (group -> member
// ids -> values) and by the scattered 4-byte accesses, not by bandwidth.
// Groups of two and of four members (on a box mesh: the nodes inside element
// faces and along element edges, 97 % of the shared nodes) come as packed
// member ids, one 8- or 16-byte load per group; the other groups keep the CSR
// (offsets -> ids -> values).  The groups are cut, in CSR order, into chunks
// of nekb_ogs::kGsChunk groups, one CTA per chunk, so the face, edge and corner
// nodes of the same elements are summed together and share sectors.  Each
// thread takes kGsGroups groups at a time and issues the loads of all of them
// before it sums.
constexpr int kGsGroups = 4, kGsThreads = 256;

struct GsGroups {
  int64_t Nchunks;
  const int32_t* chunks;  // first pair, quad and other group of chunk c at 3 c
  const int2* pairs;
  const int4* quads;
  const int32_t* offsets;
  const int32_t* ids;
};

template <typename T>
__global__ void __launch_bounds__(kGsThreads) k_gs_add(GsGroups g, int k, int64_t stride, T* __restrict__ q,
                                                       const int* skip)
{
  if (skip != nullptr && *skip != 0) return;
  const int tid = threadIdx.x;
  constexpr int kStep = kGsThreads;
  for (int64_t c = blockIdx.x; c < g.Nchunks; c += gridDim.x) {
    const int32_t* ch = g.chunks + 3 * c;
    const int32_t p_lo = ch[0], p_hi = ch[3], q_lo = ch[1], q_hi = ch[4], o_lo = ch[2], o_hi = ch[5];
    for (int f = 0; f < k; ++f) {
      T* qf = q + f * stride;
      for (int32_t p0 = p_lo + tid; p0 < p_hi; p0 += kGsGroups * kStep) {
        int2 m[kGsGroups];
#pragma unroll
        for (int u = 0; u < kGsGroups; ++u) {
          const int32_t p = p0 + u * kStep;
          m[u] = p < p_hi ? g.pairs[p] : make_int2(-1, -1);
        }
        T a[kGsGroups], b[kGsGroups];
#pragma unroll
        for (int u = 0; u < kGsGroups; ++u) {
          a[u] = m[u].x >= 0 ? qf[m[u].x] : T(0);
          b[u] = m[u].x >= 0 ? qf[m[u].y] : T(0);
        }
#pragma unroll
        for (int u = 0; u < kGsGroups; ++u) {
          if (m[u].x >= 0) {
            const T sum = a[u] + b[u];  // (0 + a) + b: the CSR-order sum
            qf[m[u].x] = sum;
            qf[m[u].y] = sum;
          }
        }
      }
      for (int32_t p0 = q_lo + tid; p0 < q_hi; p0 += kGsGroups * kStep) {
        int4 m[kGsGroups];
#pragma unroll
        for (int u = 0; u < kGsGroups; ++u) {
          const int32_t p = p0 + u * kStep;
          m[u] = p < q_hi ? g.quads[p] : make_int4(-1, -1, -1, -1);
        }
        T v[kGsGroups][4];
#pragma unroll
        for (int u = 0; u < kGsGroups; ++u) {
          const bool on = m[u].x >= 0;
          v[u][0] = on ? qf[m[u].x] : T(0);
          v[u][1] = on ? qf[m[u].y] : T(0);
          v[u][2] = on ? qf[m[u].z] : T(0);
          v[u][3] = on ? qf[m[u].w] : T(0);
        }
#pragma unroll
        for (int u = 0; u < kGsGroups; ++u) {
          if (m[u].x >= 0) {
            const T sum = ((v[u][0] + v[u][1]) + v[u][2]) + v[u][3];
            qf[m[u].x] = sum;
            qf[m[u].y] = sum;
            qf[m[u].z] = sum;
            qf[m[u].w] = sum;
          }
        }
      }
      for (int32_t g0 = o_lo + tid; g0 < o_hi; g0 += kGsGroups * kStep) {
        int32_t st[kGsGroups], en[kGsGroups], i0[kGsGroups], i1[kGsGroups];
#pragma unroll
        for (int u = 0; u < kGsGroups; ++u) {
          const int32_t gid = g0 + u * kStep;
          st[u] = en[u] = 0;
          if (gid < o_hi) {
            st[u] = g.offsets[gid];
            en[u] = g.offsets[gid + 1];
          }
        }
#pragma unroll
        for (int u = 0; u < kGsGroups; ++u) {
          i0[u] = st[u] < en[u] ? g.ids[st[u]] : -1;
          i1[u] = st[u] + 1 < en[u] ? g.ids[st[u] + 1] : -1;
        }
        T sm[kGsGroups];
#pragma unroll
        for (int u = 0; u < kGsGroups; ++u) {
          const T a = i0[u] >= 0 ? qf[i0[u]] : T(0);
          const T b = i1[u] >= 0 ? qf[i1[u]] : T(0);
          sm[u] = a + b;  // (0 + a) + b: the CSR-order sum of the first two members
        }
#pragma unroll
        for (int u = 0; u < kGsGroups; ++u)
          for (int32_t n = st[u] + 2; n < en[u]; ++n) sm[u] += qf[g.ids[n]];
#pragma unroll
        for (int u = 0; u < kGsGroups; ++u) {
          if (i0[u] >= 0) qf[i0[u]] = sm[u];
          if (i1[u] >= 0) qf[i1[u]] = sm[u];
          for (int32_t n = st[u] + 2; n < en[u]; ++n) qf[g.ids[n]] = sm[u];
        }
      }
    }
  }
}

template <typename T>
__global__ void k_mask(int64_t Nmasked, const int32_t* __restrict__ ids, int k, int64_t stride,
                       T* __restrict__ q, const int* skip)
{
  if (skip != nullptr && *skip != 0) return;
  const int64_t total = Nmasked * k;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < total;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = n / Nmasked;
    q[f * stride + ids[n - f * Nmasked]] = T(0);
  }
}

// ------------------------------------------------------------------ vector utilities
__global__ void k_fill_uniform(double* v, int64_t n, uint64_t seed, uint64_t stream, double lo,
                               double hi)
{
  const double span = __dsub_rn(hi, lo);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double u = uniform01(seed, stream, (uint64_t)i);
    v[i] = __dadd_rn(lo, __dmul_rn(span, u));  // no contraction: matches the CPU generator
  }
}

__global__ void k_d2f(const double* a, float* b, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

__global__ void k_d2bf(const double* a, __nv_bfloat16* b, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = __float2bfloat16_rn((float)a[i]);
}

__global__ void k_scale(double* v, double alpha, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] *= alpha;
}

__global__ void k_set(double* v, double alpha, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] = alpha;
}

__global__ void k_vec_inv(double* v, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] = 1.0 / v[i];
}

Nodes1D make_nodes(int Nq, const double* r, const double* w)
{
  Nodes1D nd{};
  for (int i = 0; i < Nq; ++i) {
    nd.r[i] = r[i];
    nd.w[i] = w ? w[i] : 0.0;
  }
  return nd;
}

}  // namespace

int launch_update_jacobi(int Nq, int64_t E, int64_t offset, const int32_t* mapB, const double* ggeo,
                         const double* D, const double* lambda, int bk, double* diag, cudaStream_t s)
{
  if (Nq < kMinNq || Nq > kMaxNq) return fail(NEKB_ERR_UNSUPPORTED, "updateJacobi: Nq=%d", Nq);
  if (!bk && lambda == nullptr) return fail(NEKB_ERR_INVALID, "updateJacobi: lambda is NULL");
  const int64_t n = E * Nq * Nq * Nq;
  if (n == 0) return NEKB_OK;
  if (bk)
    k_update_jacobi<true><<<grid_for(n, 256), 256, 0, s>>>(Nq, E, offset, mapB, ggeo, D, lambda, diag);
  else
    k_update_jacobi<false><<<grid_for(n, 256), 256, 0, s>>>(Nq, E, offset, mapB, ggeo, D, lambda, diag);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int launch_geometric_factors(int Nq, int64_t E, const double* EX, const double* EY,
                             const double* EZ, const double* r1d, const double* w1d, double* ggeo,
                             cudaStream_t s)
{
  if (Nq < kMinNq || Nq > kMaxNq) return fail(NEKB_ERR_UNSUPPORTED, "geometric factors: Nq=%d", Nq);
  const int64_t n = E * Nq * Nq * Nq;
  if (n == 0) return NEKB_OK;
  k_geometric_factors<<<grid_for(n, 256), 256, 0, s>>>(Nq, E, EX, EY, EZ, make_nodes(Nq, r1d, w1d),
                                                        ggeo);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int launch_physical_nodes(int Nq, int64_t E, const double* EX, const double* EY, const double* EZ,
                          const double* r1d, double* x, double* y, double* z, cudaStream_t s)
{
  const int64_t n = E * Nq * Nq * Nq;
  if (n == 0) return NEKB_OK;
  k_physical_nodes<<<grid_for(n, 256), 256, 0, s>>>(Nq, E, EX, EY, EZ, make_nodes(Nq, r1d, nullptr),
                                                     x, y, z);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int launch_trilinear_coeffs(int64_t E, const double* EX, const double* EY, const double* EZ,
                            float* coef, cudaStream_t s)
{
  if (E == 0) return NEKB_OK;
  k_trilinear_coeffs<<<grid_for(E, 128), 128, 0, s>>>(E, EX, EY, EZ, coef);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int launch_gs_add(const nekb_ogs* ogs, int k, int64_t stride, void* q, int dtype, const int* skip,
                  cudaStream_t s)
{
  if (ogs->Nmulti == 0) return NEKB_OK;
  const GsGroups g{ogs->Nchunks, ogs->d_chunks, reinterpret_cast<const int2*>(ogs->d_pairs),
                   reinterpret_cast<const int4*>(ogs->d_quads), ogs->d_offsets, ogs->d_ids};
  const unsigned grid = (unsigned)std::min<int64_t>(ogs->Nchunks, 152 * 64);
  if (dtype == NEKB_DOUBLE)
    k_gs_add<double><<<grid, kGsThreads, 0, s>>>(g, k, stride, (double*)q, skip);
  else if (dtype == NEKB_FLOAT)
    k_gs_add<float><<<grid, kGsThreads, 0, s>>>(g, k, stride, (float*)q, skip);
  else
    return fail(NEKB_ERR_UNSUPPORTED, "gather-scatter: dtype %d", dtype);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int launch_mask(int64_t Nmasked, const int32_t* ids, int k, int64_t stride, void* q, int dtype,
                const int* skip, cudaStream_t s)
{
  const int64_t n = Nmasked * k;
  if (n == 0) return NEKB_OK;
  if (dtype == NEKB_DOUBLE)
    k_mask<double><<<grid_for(n, 256), 256, 0, s>>>(Nmasked, ids, k, stride, (double*)q, skip);
  else if (dtype == NEKB_FLOAT)
    k_mask<float><<<grid_for(n, 256), 256, 0, s>>>(Nmasked, ids, k, stride, (float*)q, skip);
  else
    return fail(NEKB_ERR_UNSUPPORTED, "mask: dtype %d", dtype);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int launch_fill_uniform(double* v, int64_t n, uint64_t seed, uint64_t stream, double lo, double hi,
                        cudaStream_t s)
{
  if (n == 0) return NEKB_OK;
  k_fill_uniform<<<grid_for(n, 256), 256, 0, s>>>(v, n, seed, stream, lo, hi);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int launch_convert_d2f(const double* a, float* b, int64_t n, cudaStream_t s)
{
  if (n == 0) return NEKB_OK;
  k_d2f<<<grid_for(n, 256), 256, 0, s>>>(a, b, n);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int launch_convert_d2bf(const double* a, __nv_bfloat16* b, int64_t n, cudaStream_t s)
{
  if (n == 0) return NEKB_OK;
  k_d2bf<<<grid_for(n, 256), 256, 0, s>>>(a, b, n);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int launch_scale(double* v, double alpha, int64_t n, cudaStream_t s)
{
  if (n == 0) return NEKB_OK;
  k_scale<<<grid_for(n, 256), 256, 0, s>>>(v, alpha, n);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int launch_set_scalar(double* v, double alpha, int64_t n, cudaStream_t s)
{
  if (n == 0) return NEKB_OK;
  k_set<<<grid_for(n, 256), 256, 0, s>>>(v, alpha, n);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

int launch_vec_inv(double* v, int64_t n, cudaStream_t s)
{
  if (n == 0) return NEKB_OK;
  k_vec_inv<<<grid_for(n, 256), 256, 0, s>>>(v, n);
  NEKB_CUDA(cudaGetLastError());
  return NEKB_OK;
}

}  // namespace nekb
