// extern "C" entry points of libnekb_gb300.so (declared in include/nekb.h).
// Argument checking and status codes live here; the work is in the kernels.
#include <cstring>
#include <mutex>
#include <string>

#include "bp.h"

int nekb_ogs_build(nekb_ogs* o, int64_t N, const int64_t* ids);
void nekb_ogs_release(nekb_ogs* o);
nekb_bp* nekb_bp_create(const nekb_bp_config* cfg, void* stream, int* status);
nekb_bp* nekb_bp_create_mesh(int N, int64_t E, int Nfields, const double* ggeo, const int64_t* ids,
                             int64_t Nmasked, const int32_t* maskIds, const double* EX,
                             const double* EY, const double* EZ, void* stream, int* status);
void nekb_bp_destroy(nekb_bp* bp);

namespace nekb {
const char* last_error();
OpView make_op(nekb_bp* bp, int bk, int precision, const void* lambda);
int prepare_inner(nekb_bp* bp, int precision, int bk, const double* lambda, bool jacobi);
int bp_pcg(nekb_bp* bp, const double* lambda, double* r, double* x, double tol, int maxit,
           const nekb_pcg_opts* opts, nekb_pcg_stats* stats);
int peak_fma(int fp64, double* tflops);
int peak_copy(double* gbs);
int bp_weighted_inner_product(nekb_bp* bp, const double* w, const double* a, const double* b,
                              bool two, double* host_out);
int bp_zero_mean(nekb_bp* bp, double* q);
}  // namespace nekb

using namespace nekb;

namespace {
// GLL nodes/weights per order, for the trilinear-geometry operator
struct NodeCache {
  std::mutex mu;
  bool have[kMaxNq + 1] = {};
  float r[kMaxNq + 1][kMaxNq] = {};
  float w[kMaxNq + 1][kMaxNq] = {};
} g_nodes;

int fill_nodes(int Nq, AxArgs& a)
{
  std::lock_guard<std::mutex> lk(g_nodes.mu);
  if (!g_nodes.have[Nq]) {
    double r[kMaxNq], w[kMaxNq];
    NEKB_TRY(gll_nodes(Nq - 1, r, w));
    for (int i = 0; i < Nq; ++i) {
      g_nodes.r[Nq][i] = (float)r[i];
      g_nodes.w[Nq][i] = (float)w[i];
    }
    g_nodes.have[Nq] = true;
  }
  for (int i = 0; i < Nq; ++i) {
    a.r1d[i] = g_nodes.r[Nq][i];
    a.w1d[i] = g_nodes.w[Nq][i];
  }
  return NEKB_OK;
}
}  // namespace

extern "C" {

const char* nekb_last_error(void) { return last_error(); }

int nekb_version(void) { return 10000; }

int nekb_device_sync(void)
{
  NEKB_CUDA(cudaDeviceSynchronize());
  return NEKB_OK;
}

int nekb_copy(void* dst, const void* src, int64_t bytes)
{
  if (bytes < 0 || (bytes > 0 && (!dst || !src))) return fail(NEKB_ERR_INVALID, "copy: bad arguments");
  if (bytes == 0) return NEKB_OK;
  NEKB_CUDA(cudaMemcpy(dst, src, (size_t)bytes, cudaMemcpyDefault));
  return NEKB_OK;
}

int nekb_axhelm(int Nq, int flags, int precision, int64_t Nelements, int64_t offset,
                const int32_t* elementList, const void* ggeo, const void* D, const void* lambda,
                const void* q, void* Aq, void* stream)
{
  if (Nelements < 0) return fail(NEKB_ERR_INVALID, "axhelm: Nelements=%lld", (long long)Nelements);
  if (Nelements == 0) return NEKB_OK;
  if (!ggeo || !D || !q || !Aq) return fail(NEKB_ERR_INVALID, "axhelm: NULL array");
  if ((flags & NEKB_AX_PARTIAL) && !elementList)
    return fail(NEKB_ERR_INVALID, "axhelm: Partial variant needs an element list");
  if (!(flags & NEKB_AX_BK) && !lambda) return fail(NEKB_ERR_INVALID, "axhelm: lambda is NULL outside BK mode");
  if (Nq < kMinNq || Nq > kMaxNq) return fail(NEKB_ERR_UNSUPPORTED, "axhelm: Nq=%d outside 2..%d", Nq, kMaxNq);
  const int64_t Np = (int64_t)Nq * Nq * Nq;
  const int64_t nf = (flags & NEKB_AX_N3) ? 3 : 1;
  if (!(flags & NEKB_AX_PARTIAL) && offset < Nelements * Np)
    return fail(NEKB_ERR_INVALID, "axhelm: offset %lld < Nelements*Np", (long long)offset);
  if (nf > 1 && offset <= 0) return fail(NEKB_ERR_INVALID, "axhelm: n3 needs offset > 0");
  AxArgs a{};
  a.Nelements = Nelements;
  a.offset = offset;
  a.elementList = elementList;
  a.ggeo = ggeo;
  a.D = D;
  a.lambda = lambda;
  a.q = q;
  a.Aq = Aq;
  a.skip = nullptr;
  if (precision == NEKB_FP32_TRILINEAR) NEKB_TRY(fill_nodes(Nq, a));
  return launch_axhelm(Nq, flags, precision, a, static_cast<cudaStream_t>(stream));
}

int nekb_axhelm_flags_from_name(const char* name, int* flags)
{
  if (!name || !flags) return fail(NEKB_ERR_INVALID, "axhelm name: NULL argument");
  if (std::strncmp(name, "axhelm", 6) != 0) return fail(NEKB_ERR_INVALID, "axhelm name '%s'", name);
  const char* p = name + 6;
  int f = 0;
  if (std::strncmp(p, "Partial", 7) == 0) {
    f |= NEKB_AX_PARTIAL;
    p += 7;
  } else if (std::strncmp(p, "_partial", 8) == 0) {  // spelling used by axhelm/main.cpp:106
    f |= NEKB_AX_PARTIAL;
    p += 8;
  }
  if (std::strncmp(p, "_bk", 3) == 0) {
    f |= NEKB_AX_BK;
    p += 3;
  }
  if (std::strncmp(p, "_n3", 3) == 0) {
    f |= NEKB_AX_N3;
    p += 3;
  }
  if (std::strncmp(p, "_v", 2) != 0 || p[2] < '0' || p[2] > '9')
    return fail(NEKB_ERR_INVALID, "axhelm name '%s': expected _v<id> suffix", name);
  *flags = f;
  return NEKB_OK;
}

int nekb_update_jacobi(int Nq, int64_t Nelements, int64_t offset, const int32_t* mapB,
                       const double* ggeo, const double* D, const double* lambda, double* diag,
                       void* stream)
{
  if (!ggeo || !D || !diag || !lambda) return fail(NEKB_ERR_INVALID, "updateJacobi: NULL array");
  return launch_update_jacobi(Nq, Nelements, offset, mapB, ggeo, D, lambda, 0, diag,
                              static_cast<cudaStream_t>(stream));
}

int nekb_geometric_factors(int Nq, int64_t Nelements, const double* EX, const double* EY,
                           const double* EZ, const double* r1d, const double* w1d, double* ggeo,
                           void* stream)
{
  if (!EX || !EY || !EZ || !r1d || !w1d || !ggeo) return fail(NEKB_ERR_INVALID, "geometric factors: NULL");
  return launch_geometric_factors(Nq, Nelements, EX, EY, EZ, r1d, w1d, ggeo,
                                  static_cast<cudaStream_t>(stream));
}

int nekb_trilinear_coeffs(int64_t Nelements, const double* EX, const double* EY, const double* EZ,
                          float* coef, void* stream)
{
  if (!EX || !EY || !EZ || !coef) return fail(NEKB_ERR_INVALID, "trilinear coefficients: NULL");
  return launch_trilinear_coeffs(Nelements, EX, EY, EZ, coef, static_cast<cudaStream_t>(stream));
}

int nekb_gll(int N, double* r, double* w)
{
  if (!r || !w) return fail(NEKB_ERR_INVALID, "gll: NULL");
  return gll_nodes(N, r, w);
}

int nekb_gauss(int N, double* r, double* w)
{
  if (!r || !w) return fail(NEKB_ERR_INVALID, "gauss: NULL");
  return gauss_nodes(N, r, w);
}

int nekb_dmatrix(int Nq, const double* r, double* D)
{
  if (!r || !D || Nq < 1 || Nq > 64) return fail(NEKB_ERR_INVALID, "dmatrix: bad arguments");
  deriv_matrix(Nq, r, D);
  return NEKB_OK;
}

int nekb_fill_uniform(double* v, int64_t n, uint64_t seed, uint64_t stream, double lo, double hi,
                      void* stream_)
{
  if (n < 0 || (n > 0 && !v)) return fail(NEKB_ERR_INVALID, "fill_uniform: bad arguments");
  return launch_fill_uniform(v, n, seed, stream, lo, hi, static_cast<cudaStream_t>(stream_));
}

// ------------------------------------------------------------------ ogs
nekb_ogs* nekb_ogs_setup(int64_t N, const int64_t* ids, int verbose, int* status)
{
  (void)verbose;
  int st = NEKB_OK;
  nekb_ogs* o = nullptr;
  if (N < 0 || (N > 0 && !ids)) {
    st = fail(NEKB_ERR_INVALID, "ogsSetup: bad arguments");
  } else if (N > INT32_MAX) {
    st = fail(NEKB_ERR_INVALID, "ogsSetup: N=%lld exceeds 32-bit local ids", (long long)N);
  } else {
    o = new nekb_ogs();
    st = nekb_ogs_build(o, N, ids);
    if (st != NEKB_OK) {
      nekb_ogs_release(o);
      o = nullptr;
    }
  }
  if (status) *status = st;
  return o;
}

void nekb_ogs_free(nekb_ogs* ogs) { nekb_ogs_release(ogs); }

int nekb_ogs_gs_many(nekb_ogs* ogs, void* v, int k, int64_t stride, int dtype, int op, void* stream)
{
  if (!ogs) return fail(NEKB_ERR_INVALID, "gs: NULL handle");
  if (op != NEKB_OP_ADD) return fail(NEKB_ERR_UNSUPPORTED, "gs: only the add operation is supported");
  if (k < 1 || (k > 1 && stride < ogs->N)) return fail(NEKB_ERR_INVALID, "gs: k=%d stride=%lld", k, (long long)stride);
  if (!v && ogs->Nmulti > 0) return fail(NEKB_ERR_INVALID, "gs: NULL vector");
  return launch_gs_add(ogs, k, stride, v, dtype, nullptr, static_cast<cudaStream_t>(stream));
}

int nekb_ogs_sizes(const nekb_ogs* ogs, int64_t* s)
{
  if (!ogs || !s) return fail(NEKB_ERR_INVALID, "ogs sizes: NULL");
  s[0] = ogs->N;
  s[1] = ogs->Nlocal;
  s[2] = ogs->NlocalGather;
  s[3] = ogs->Nmulti;
  return NEKB_OK;
}

int nekb_ogs_copy_csr(const nekb_ogs* ogs, int32_t* offsets, int32_t* ids)
{
  if (!ogs || !offsets || !ids) return fail(NEKB_ERR_INVALID, "ogs csr: NULL");
  std::memcpy(offsets, ogs->h_offsets.data(), sizeof(int32_t) * ogs->h_offsets.size());
  std::memcpy(ids, ogs->h_ids.data(), sizeof(int32_t) * ogs->h_ids.size());
  return NEKB_OK;
}

const double* nekb_ogs_inv_degree(const nekb_ogs* ogs) { return ogs ? ogs->d_invDegree : nullptr; }

int nekb_mask(int64_t Nmasked, const int32_t* maskIds, void* q, int dtype, void* stream)
{
  if (Nmasked < 0 || (Nmasked > 0 && (!maskIds || !q))) return fail(NEKB_ERR_INVALID, "mask: bad arguments");
  return launch_mask(Nmasked, maskIds, 1, 0, q, dtype, nullptr, static_cast<cudaStream_t>(stream));
}

// ------------------------------------------------------------------ benchmark problem
nekb_bp* nekb_bp_setup(const nekb_bp_config* cfg, void* stream, int* status)
{
  return nekb_bp_create(cfg, stream, status);
}

nekb_bp* nekb_bp_setup_mesh(int N, int64_t Nelements, int Nfields, const double* ggeo,
                            const int64_t* ids, int64_t Nmasked, const int32_t* maskIds,
                            const double* EX, const double* EY, const double* EZ, void* stream,
                            int* status)
{
  return nekb_bp_create_mesh(N, Nelements, Nfields, ggeo, ids, Nmasked, maskIds, EX, EY, EZ,
                             stream, status);
}

void nekb_bp_free(nekb_bp* bp) { nekb_bp_destroy(bp); }

int nekb_bp_sizes(const nekb_bp* bp, int64_t* s)
{
  if (!bp || !s) return fail(NEKB_ERR_INVALID, "bp sizes: NULL");
  s[0] = bp->Nq;
  s[1] = bp->E;
  s[2] = bp->Np;
  s[3] = bp->offset;
  s[4] = bp->Nmasked;
  s[5] = bp->Nfields;
  return NEKB_OK;
}

void* nekb_bp_device_ptr(nekb_bp* bp, const char* name)
{
  if (!bp || !name) return nullptr;
  const std::string n(name);
  if (n == "ggeo") return bp->ggeo.p;
  if (n == "D") return bp->D.p;
  if (n == "Df") return bp->Df.p;
  if (n == "invDegree") return bp->ogs->d_invDegree;
  if (n == "maskIds") return bp->mask.p;
  if (n == "EX") return bp->EX.p;
  if (n == "EY") return bp->EY.p;
  if (n == "EZ") return bp->EZ.p;
  if (n == "trilinear") return bp->tri.p;
  if (n == "invDiag") return bp->invDiag.p;
  if (n == "x" || n == "y" || n == "z") {
    if (bp->EX.p == nullptr) {
      fail(NEKB_ERR_UNSUPPORTED, "bp device ptr: node coordinates need the element vertices");
      return nullptr;
    }
    const int64_t Nl = bp->Nlocal;
    if (bp->xyz.p == nullptr) {
      if (bp->xyz.ensure(sizeof(double) * 3 * Nl) != NEKB_OK) return nullptr;
      double* b = bp->xyz.as<double>();
      if (launch_physical_nodes(bp->Nq, bp->E, bp->EX.as<double>(), bp->EY.as<double>(),
                                bp->EZ.as<double>(), bp->r1d, b, b + Nl, b + 2 * Nl, bp->stream) != NEKB_OK)
        return nullptr;
      if (cudaStreamSynchronize(bp->stream) != cudaSuccess) return nullptr;
    }
    return bp->xyz.as<double>() + (n == "x" ? 0 : n == "y" ? Nl : 2 * Nl);
  }
  if (n == "ggeo_f") return prepare_inner(bp, NEKB_FP32, 1, nullptr, false) == NEKB_OK ? bp->ggeo_f.p : nullptr;
  if (n == "ggeo_bf") return prepare_inner(bp, NEKB_BF16, 1, nullptr, false) == NEKB_OK ? bp->ggeo_bf.p : nullptr;
  fail(NEKB_ERR_INVALID, "bp device ptr: unknown name '%s'", name);
  return nullptr;
}

nekb_ogs* nekb_bp_ogs(nekb_bp* bp) { return bp ? bp->ogs : nullptr; }

int nekb_bp_apply(nekb_bp* bp, int bk, int precision, const void* lambda, const void* q, void* Aq)
{
  if (!bp || !q || !Aq) return fail(NEKB_ERR_INVALID, "bp apply: NULL argument");
  if (!bk && !lambda) return fail(NEKB_ERR_INVALID, "bp apply: lambda is NULL");
  if (precision == NEKB_FP32_TRILINEAR && bp->tri.p == nullptr)
    return fail(NEKB_ERR_UNSUPPORTED, "bp apply: trilinear geometry needs the element vertices");
  if (precision != NEKB_FP64 && precision != NEKB_FP64_SPLIT)
    NEKB_TRY(prepare_inner(bp, precision, 1, nullptr, false));
  OpView op = make_op(bp, bk, precision, lambda);
  NEKB_TRY(apply_op(op, q, Aq, nullptr, bp->stream));
  NEKB_CUDA(cudaStreamSynchronize(bp->stream));
  return NEKB_OK;
}

int nekb_bp_weighted_inner_product(nekb_bp* bp, const double* w, const double* a, const double* b,
                                   double* wab)
{
  return bp_weighted_inner_product(bp, w, a, b, false, wab);
}

int nekb_bp_weighted_inner_product2(nekb_bp* bp, const double* w, const double* a,
                                    const double* b, double* wab2)
{
  return bp_weighted_inner_product(bp, w, a, b, true, wab2);
}

void nekb_pcg_default_opts(nekb_pcg_opts* o)
{
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->solver = NEKB_SOLVER_FP64;
  o->precond = NEKB_PRECOND_JACOBI;
  o->inner_precision = NEKB_FP32;
  o->inner_tol = 1e-2;
  o->max_outer = 20;
  o->check_every = 16;
  o->use_graph = 1;
}

int nekb_bp_zero_mean(nekb_bp* bp, double* q)
{
  NEKB_TRY(bp_zero_mean(bp, q));
  NEKB_CUDA(cudaStreamSynchronize(bp->stream));
  return NEKB_OK;
}

int nekb_bp_pcg(nekb_bp* bp, const double* lambda, double* r, double* x, double tol, int maxit,
                const nekb_pcg_opts* opts, nekb_pcg_stats* stats)
{
  return bp_pcg(bp, lambda, r, x, tol, maxit, opts, stats);
}

int nekb_peak_fma(int fp64, double* tflops)
{
  if (!tflops) return fail(NEKB_ERR_INVALID, "peak: NULL");
  return peak_fma(fp64, tflops);
}

int nekb_peak_copy(double* gbs)
{
  if (!gbs) return fail(NEKB_ERR_INVALID, "peak: NULL");
  return peak_copy(gbs);
}

}  // extern "C"
