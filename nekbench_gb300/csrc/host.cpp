// Host-side pieces of the library: error state, 1D basis and the
// gather-scatter setup (index/ownership work done once, on the CPU, like the
// reference's ogsSetup).
#include "internal.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>

namespace nekb {

// ------------------------------------------------------------------ errors
static thread_local char g_err[512] = "";

int fail(int code, const char* fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line)
{
  const char* base = strrchr(file, '/');
  snprintf(g_err, sizeof(g_err), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e),
           base ? base + 1 : file, line);
  return e == cudaErrorMemoryAllocation ? NEKB_ERR_ALLOC : NEKB_ERR_CUDA;
}

void clear_error() { g_err[0] = 0; }
const char* last_error() { return g_err; }

// ------------------------------------------------------------------ 1D basis
// Nodes by Newton iteration on the Legendre three-term recurrence (nodes of
// meshJacobiGL/meshJacobiGQ, core/meshBasis.cpp:46-173), derivative matrix by
// the barycentric formula (the matrix meshDmatrix1D, :775-786, builds by a
// Vandermonde solve).  Nodes are made exactly antisymmetric about 0, which
// makes D centro-antisymmetric.
static void legendre_pair(int n, double x, double& p, double& dp)
{
  double p0 = 1.0, p1 = x, d0 = 0.0, d1 = 1.0;
  if (n == 0) { p = 1.0; dp = 0.0; return; }
  for (int k = 2; k <= n; ++k) {
    const double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
    const double d2 = d0 + (2 * k - 1) * p1;
    p0 = p1; p1 = p2; d0 = d1; d1 = d2;
  }
  p = p1; dp = d1;
}

int gll_nodes(int N, double* r, double* w)
{
  if (N < 1 || N > kMaxNq - 1) return fail(NEKB_ERR_UNSUPPORTED, "GLL: N=%d outside 1..%d", N, kMaxNq - 1);
  const double pi = 3.14159265358979323846;
  r[0] = -1.0;
  r[N] = 1.0;
  for (int j = 1; j <= N / 2; ++j) {
    // interior GLL nodes: zeros of L_N'; Newton on (L_{N+1} - L_{N-1}) = (2N+1) int L_N
    double x = -std::cos(pi * j / N);
    for (int it = 0; it < 100; ++it) {
      double a, da, b, db;
      legendre_pair(N + 1, x, a, da);
      legendre_pair(N - 1, x, b, db);
      const double dx = (a - b) / (da - db);
      x -= dx;
      if (std::fabs(dx) < 1e-16 * (1 + std::fabs(x))) break;
    }
    r[j] = x;
    r[N - j] = -x;
  }
  if (N % 2 == 0) r[N / 2] = 0.0;
  for (int j = 0; j <= N; ++j) {
    double p, dp;
    legendre_pair(N, r[j], p, dp);
    w[j] = 2.0 / (N * (N + 1.0) * p * p);
  }
  return NEKB_OK;
}

int gauss_nodes(int N, double* r, double* w)
{
  if (N < 0 || N > kMaxNq - 1) return fail(NEKB_ERR_UNSUPPORTED, "Gauss: N=%d outside 0..%d", N, kMaxNq - 1);
  const double pi = 3.14159265358979323846;
  const int n = N + 1;
  for (int j = 0; j < (n + 1) / 2; ++j) {
    double x = -std::cos(pi * (2 * j + 1) / (2.0 * n));
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre_pair(n, x, p, dp);
      const double dx = p / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-16 * (1 + std::fabs(x))) break;
    }
    r[j] = x;
    r[n - 1 - j] = -x;
  }
  if (n % 2 == 1) r[n / 2] = 0.0;
  for (int j = 0; j < n; ++j) {
    double p, dp;
    legendre_pair(n, r[j], p, dp);
    w[j] = 2.0 / ((1.0 - r[j] * r[j]) * dp * dp);
  }
  return NEKB_OK;
}

void deriv_matrix(int Nq, const double* r, double* D)
{
  std::vector<double> lam(Nq);
  for (int j = 0; j < Nq; ++j) {
    double p = 1.0;
    for (int k = 0; k < Nq; ++k)
      if (k != j) p *= r[j] - r[k];
    lam[j] = 1.0 / p;
  }
  for (int i = 0; i < Nq; ++i) {
    double s = 0.0;
    for (int j = 0; j < Nq; ++j) {
      if (j == i) continue;
      const double d = lam[j] / (lam[i] * (r[i] - r[j]));
      D[i * Nq + j] = d;
      s += d;
    }
    D[i * Nq + i] = -s;
  }
}

}  // namespace nekb

// ------------------------------------------------------------------ gather-scatter setup
// Restates the local branch of ogsSetup (3rdParty/ogs/src/ogsSetup.cpp:137-212)
// and the degree vector (:325-352) with linear-time passes:
//  1. nodes with id != 0 are ordered by |id| with a stable counting sort (a
//     stable comparison sort when ids are sparse), so nodes of equal |id|
//     stay in ascending local index: the (|id|, localId) order of the
//     reference's qsort (:40-54, 156);
//  2. a group is a run of equal SIGNED id in that order: the reference opens
//     a new gather node whenever the signed id differs from its predecessor
//     (:161-166), so ids 5,-5,5 at local indices 0,1,2 make three groups;
//  3. groups are numbered by the local index of their first member, which is
//     the order the reference's re-sort by local id produces (:173-189);
//  4. CSR offsets/ids in that order; invDegree = 1/size (1 for id-0 nodes).
// The result is bit-identical to the reference CSR for any id array, signed
// ids included.
int nekb_ogs_build(nekb_ogs* o, int64_t N, const int64_t* ids)
{
  using namespace nekb;
  o->N = N;
  std::vector<int64_t> key;  // |id| of nonzero nodes, in local order
  std::vector<int32_t> lid;
  key.reserve(N);
  lid.reserve(N);
  int64_t kmin = INT64_MAX, kmax = 0;
  for (int64_t i = 0; i < N; ++i) {
    if (ids[i] == 0) continue;
    const int64_t a = ids[i] < 0 ? -ids[i] : ids[i];
    key.push_back(a);
    lid.push_back((int32_t)i);
    kmin = std::min(kmin, a);
    kmax = std::max(kmax, a);
  }
  const int64_t Nl = (int64_t)key.size();
  o->Nlocal = Nl;
  std::vector<int32_t> order(Nl);  // positions into key/lid, grouped by key, stable
  if (Nl > 0 && (kmax - kmin) <= 4 * Nl + 1024) {
    const int64_t R = kmax - kmin + 1;
    std::vector<int64_t> cnt(R + 1, 0);
    for (int64_t p = 0; p < Nl; ++p) cnt[key[p] - kmin + 1]++;
    for (int64_t b = 0; b < R; ++b) cnt[b + 1] += cnt[b];
    for (int64_t p = 0; p < Nl; ++p) order[cnt[key[p] - kmin]++] = (int32_t)p;
  } else {
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t a, int32_t b) { return key[a] < key[b]; });
  }
  // runs of equal signed id: run r spans order[rs[r] .. rs[r+1])
  std::vector<int64_t> rs;
  rs.reserve(Nl / 2 + 2);
  for (int64_t p = 0; p < Nl; ++p)
    if (p == 0 || ids[lid[order[p]]] != ids[lid[order[p - 1]]]) rs.push_back(p);
  rs.push_back(Nl);
  const int64_t Ng = (int64_t)rs.size() - 1;
  o->NlocalGather = Ng;
  // number groups by their first (lowest) local index
  std::vector<int32_t> run_at(N, -1);
  for (int64_t r = 0; r < Ng; ++r) run_at[lid[order[rs[r]]]] = (int32_t)r;
  std::vector<int32_t> final_of(Ng);
  int64_t g = 0;
  for (int64_t i = 0; i < N; ++i)
    if (run_at[i] >= 0) final_of[run_at[i]] = (int32_t)g++;
  std::vector<int32_t>().swap(run_at);
  std::vector<int64_t> size(Ng);
  for (int64_t r = 0; r < Ng; ++r) size[final_of[r]] = rs[r + 1] - rs[r];
  o->h_offsets.assign(Ng + 1, 0);
  for (int64_t q = 0; q < Ng; ++q) o->h_offsets[q + 1] = (int32_t)(o->h_offsets[q] + size[q]);
  o->h_ids.assign(Nl, 0);
  for (int64_t r = 0; r < Ng; ++r) {
    const int32_t base = o->h_offsets[final_of[r]];
    for (int64_t p = rs[r]; p < rs[r + 1]; ++p) o->h_ids[base + (p - rs[r])] = lid[order[p]];
  }
  // degree vector
  std::vector<double> invdeg(N, 1.0);
  for (int64_t q = 0; q < Ng; ++q) {
    const int32_t s = o->h_offsets[q], e = o->h_offsets[q + 1];
    const double v = 1.0 / (double)(e - s);
    for (int32_t n = s; n < e; ++n) invdeg[o->h_ids[n]] = v;
  }
  // the groups with more than one member, for the device kernel: in CSR
  // order, chunks of kGsChunk groups (a chunk's nodes lie close together, so
  // one CTA's loads share sectors), each split into groups of two and of four
  // (packed member ids) and the others (a compact CSR)
  std::vector<int32_t> pairs, quads, moff(1, 0), mids, chunks;
  int64_t nm = 0;
  for (int64_t q = 0; q < Ng; ++q) {
    const int32_t s = o->h_offsets[q], e = o->h_offsets[q + 1];
    if (e - s < 2) continue;
    if (nm++ % nekb_ogs::kGsChunk == 0) {
      chunks.push_back((int32_t)(pairs.size() / 2));
      chunks.push_back((int32_t)(quads.size() / 4));
      chunks.push_back((int32_t)(moff.size() - 1));
    }
    std::vector<int32_t>& dst = e - s == 2 ? pairs : (e - s == 4 ? quads : mids);
    for (int32_t n = s; n < e; ++n) dst.push_back(o->h_ids[n]);
    if (e - s != 2 && e - s != 4) moff.push_back((int32_t)mids.size());
  }
  o->Npairs = (int64_t)pairs.size() / 2;
  o->Nquads = (int64_t)quads.size() / 4;
  o->Nrest = (int64_t)moff.size() - 1;
  o->Nmulti = o->Npairs + o->Nquads + o->Nrest;
  o->Nchunks = (int64_t)chunks.size() / 3;
  chunks.push_back((int32_t)o->Npairs);
  chunks.push_back((int32_t)o->Nquads);
  chunks.push_back((int32_t)o->Nrest);
  auto upload = [](int32_t** d, const std::vector<int32_t>& h) -> int {
    if (h.empty()) return NEKB_OK;
    NEKB_CUDA(cudaMalloc(d, sizeof(int32_t) * h.size()));
    NEKB_CUDA(cudaMemcpy(*d, h.data(), sizeof(int32_t) * h.size(), cudaMemcpyHostToDevice));
    return NEKB_OK;
  };
  NEKB_TRY(upload(&o->d_chunks, chunks));
  NEKB_TRY(upload(&o->d_pairs, pairs));
  NEKB_TRY(upload(&o->d_quads, quads));
  NEKB_TRY(upload(&o->d_offsets, moff));
  NEKB_TRY(upload(&o->d_ids, mids));
  if (N > 0) {
    NEKB_CUDA(cudaMalloc(&o->d_invDegree, sizeof(double) * N));
    NEKB_CUDA(cudaMemcpy(o->d_invDegree, invdeg.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
  }
  return NEKB_OK;
}
