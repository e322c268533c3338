// Benchmark problem: structured box mesh of perturbed trilinear hexahedra,
// geometric factors, gather-scatter handle, Dirichlet mask and workspace.
// Mesh semantics follow meshSetupBoxHex3D (core/meshSetup.cpp:2265-2451):
// element e = ex + nx*(ey + ny*ez), vertex order of :2363-2410, global node
// numbering on the (nx*N+1)x(ny*N+1)x(nz*N+1) lattice (modulo nx*N when
// periodic, as :2363-2376).  The reference's box is periodic and unperturbed;
// the Dirichlet/perturbed form is the one the benchmark configurations use.
#include "bp.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

int nekb_ogs_build(nekb_ogs* o, int64_t N, const int64_t* ids);
void nekb_ogs_release(nekb_ogs* o);
void nekb_bp_destroy(nekb_bp* bp);

namespace nekb {

int DeviceBuf::ensure(size_t b)
{
  if (b <= bytes && p != nullptr) return NEKB_OK;
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
  if (b == 0) return NEKB_OK;
  NEKB_CUDA(cudaMalloc(&p, b));
  bytes = b;
  return NEKB_OK;
}

DeviceBuf::~DeviceBuf()
{
  if (p) cudaFree(p);
}

int apply_op(const OpView& op, const void* q, void* Aq, const int* skip, cudaStream_t s,
             double* dot_partials, int* dot_count)
{
  AxArgs a{};
  a.dot_partials = dot_partials;
  a.dot_count = dot_count;
  a.Nelements = op.E;
  a.offset = op.offset;
  a.elementList = nullptr;
  a.ggeo = op.ggeo;
  a.D = op.D;
  a.lambda = op.lambda;
  a.q = q;
  a.Aq = Aq;
  a.skip = skip;
  for (int i = 0; i < kMaxNq; ++i) {
    a.r1d[i] = op.r1d[i];
    a.w1d[i] = op.w1d[i];
  }
  NEKB_TRY(launch_axhelm(op.Nq, op.flags, op.precision, a, s));
  const bool fp64 = op.precision == NEKB_FP64 || op.precision == NEKB_FP64_SPLIT;
  const int dtype = fp64 ? NEKB_DOUBLE : NEKB_FLOAT;
  NEKB_TRY(launch_gs_add(op.ogs, op.Nfields, op.offset, Aq, dtype, skip, s));
  NEKB_TRY(launch_mask(op.Nmasked, op.mask, op.Nfields, op.offset, Aq, dtype, skip, s));
  return NEKB_OK;
}

// host mesh: vertices (perturbed, same arithmetic as the CPU oracle), global ids, mask list
static void box_vertices(const nekb_bp_config& c, double* EX, double* EY, double* EZ)
{
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  const bool ext = c.box_max > c.box_min;
  const double lo = ext ? c.box_min : 0.0, len = ext ? c.box_max - c.box_min : 1.0;
  const double hx = len / nx, hy = len / ny, hz = len / nz;
  static const int vi[8] = {0, 1, 1, 0, 0, 1, 1, 0};
  static const int vj[8] = {0, 0, 1, 1, 0, 0, 1, 1};
  static const int vk[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  const int64_t E = (int64_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < E; ++e) {
    const int ex = (int)(e % nx), ey = (int)((e / nx) % ny), ez = (int)(e / ((int64_t)nx * ny));
    for (int v = 0; v < 8; ++v) {
      const int I = ex + vi[v], J = ey + vj[v], K = ez + vk[v];
      double X = lo + I * hx, Y = lo + J * hy, Z = lo + K * hz;
      const bool interior = I > 0 && I < nx && J > 0 && J < ny && K > 0 && K < nz;
      if (interior && !c.periodic && c.perturb != 0.0) {
        const uint64_t vid = (uint64_t)I + (uint64_t)(nx + 1) * ((uint64_t)J + (uint64_t)(ny + 1) * K);
        const double ux = uniform01(c.seed, 1, 3 * vid + 0);
        const double uy = uniform01(c.seed, 1, 3 * vid + 1);
        const double uz = uniform01(c.seed, 1, 3 * vid + 2);
        X += c.perturb * hx * (2.0 * ux - 1.0);
        Y += c.perturb * hy * (2.0 * uy - 1.0);
        Z += c.perturb * hz * (2.0 * uz - 1.0);
      }
      EX[e * 8 + v] = X;
      EY[e * 8 + v] = Y;
      EZ[e * 8 + v] = Z;
    }
  }
}

static void box_ids(const nekb_bp_config& c, int64_t* ids, std::vector<int32_t>& mask)
{
  const int N = c.N, Nq = N + 1;
  const int64_t Np = (int64_t)Nq * Nq * Nq;
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  const int64_t GX = (int64_t)nx * N + (c.periodic ? 0 : 1);
  const int64_t GY = (int64_t)ny * N + (c.periodic ? 0 : 1);
  const int64_t E = (int64_t)nx * ny * nz;
  const bool dir = c.dirichlet && !c.periodic;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < E; ++e) {
    const int64_t ex = e % nx, ey = (e / nx) % ny, ez = e / ((int64_t)nx * ny);
    for (int k = 0; k < Nq; ++k)
      for (int j = 0; j < Nq; ++j)
        for (int i = 0; i < Nq; ++i) {
          int64_t I = ex * N + i, J = ey * N + j, K = ez * N + k;
          const bool bnd = I == 0 || J == 0 || K == 0 || I == (int64_t)nx * N ||
                           J == (int64_t)ny * N || K == (int64_t)nz * N;
          if (c.periodic) {
            I %= (int64_t)nx * N;
            J %= (int64_t)ny * N;
            K %= (int64_t)nz * N;
          }
          ids[e * Np + i + Nq * (j + Nq * k)] = (dir && bnd) ? 0 : 1 + I + GX * (J + GY * K);
        }
  }
  if (dir) {
    for (int64_t e = 0; e < E; ++e) {
      const int64_t ex = e % nx, ey = (e / nx) % ny, ez = e / ((int64_t)nx * ny);
      const bool touches = ex == 0 || ey == 0 || ez == 0 || ex == nx - 1 || ey == ny - 1 || ez == nz - 1;
      if (!touches) continue;
      for (int k = 0; k < Nq; ++k)
        for (int j = 0; j < Nq; ++j)
          for (int i = 0; i < Nq; ++i) {
            const int64_t I = ex * N + i, J = ey * N + j, K = ez * N + k;
            if (I == 0 || J == 0 || K == 0 || I == (int64_t)nx * N || J == (int64_t)ny * N ||
                K == (int64_t)nz * N)
              mask.push_back((int32_t)(e * Np + i + Nq * (j + Nq * k)));
          }
    }
  }
}

static int bp_build(nekb_bp* bp, const nekb_bp_config& c, cudaStream_t user_stream)
{
  bp->cfg = c;
  bp->N = c.N;
  bp->Nq = c.N + 1;
  bp->Np = bp->Nq * bp->Nq * bp->Nq;
  bp->Nfields = c.Nfields;
  bp->E = (int64_t)c.nx * c.ny * c.nz;
  bp->Nlocal = bp->E * bp->Np;
  bp->offset = bp->Nlocal;
  if (bp->Nlocal > INT32_MAX) return fail(NEKB_ERR_INVALID, "BP: %lld local nodes exceed 32-bit ids", (long long)bp->Nlocal);
  if (user_stream) {
    bp->stream = user_stream;
  } else {
    NEKB_CUDA(cudaStreamCreateWithFlags(&bp->stream, cudaStreamNonBlocking));
    bp->own_stream = true;
  }
  NEKB_TRY(gll_nodes(c.N, bp->r1d, bp->w1d));
  const int Nq = bp->Nq;
  const int64_t E = bp->E, Nl = bp->Nlocal;
  cudaStream_t s = bp->stream;

  // vertices
  std::vector<double> hx(E * 8), hy(E * 8), hz(E * 8);
  box_vertices(c, hx.data(), hy.data(), hz.data());
  NEKB_TRY(bp->EX.ensure(sizeof(double) * E * 8));
  NEKB_TRY(bp->EY.ensure(sizeof(double) * E * 8));
  NEKB_TRY(bp->EZ.ensure(sizeof(double) * E * 8));
  NEKB_CUDA(cudaMemcpyAsync(bp->EX.p, hx.data(), sizeof(double) * E * 8, cudaMemcpyHostToDevice, s));
  NEKB_CUDA(cudaMemcpyAsync(bp->EY.p, hy.data(), sizeof(double) * E * 8, cudaMemcpyHostToDevice, s));
  NEKB_CUDA(cudaMemcpyAsync(bp->EZ.p, hz.data(), sizeof(double) * E * 8, cudaMemcpyHostToDevice, s));

  // geometry
  NEKB_TRY(bp->ggeo.ensure(sizeof(double) * 7 * Nl));
  NEKB_TRY(launch_geometric_factors(Nq, E, bp->EX.as<double>(), bp->EY.as<double>(),
                                    bp->EZ.as<double>(), bp->r1d, bp->w1d, bp->ggeo.as<double>(), s));
  NEKB_TRY(bp->tri.ensure(sizeof(float) * 24 * E));
  NEKB_TRY(launch_trilinear_coeffs(E, bp->EX.as<double>(), bp->EY.as<double>(), bp->EZ.as<double>(),
                                   bp->tri.as<float>(), s));
  std::vector<double> hD(Nq * Nq);
  deriv_matrix(Nq, bp->r1d, hD.data());
  std::vector<float> hDf(Nq * Nq);
  for (int t = 0; t < Nq * Nq; ++t) hDf[t] = (float)hD[t];
  NEKB_TRY(bp->D.ensure(sizeof(double) * Nq * Nq));
  NEKB_TRY(bp->Df.ensure(sizeof(float) * Nq * Nq));
  NEKB_CUDA(cudaMemcpyAsync(bp->D.p, hD.data(), sizeof(double) * Nq * Nq, cudaMemcpyHostToDevice, s));
  NEKB_CUDA(cudaMemcpyAsync(bp->Df.p, hDf.data(), sizeof(float) * Nq * Nq, cudaMemcpyHostToDevice, s));

  // numbering, gather-scatter, mask
  std::vector<int64_t> ids(Nl);
  std::vector<int32_t> mask;
  box_ids(c, ids.data(), mask);
  bp->ogs = new nekb_ogs();
  NEKB_TRY(nekb_ogs_build(bp->ogs, Nl, ids.data()));
  std::vector<int64_t>().swap(ids);
  bp->Nmasked = (int64_t)mask.size();
  if (!mask.empty()) {
    NEKB_TRY(bp->mask.ensure(sizeof(int32_t) * mask.size()));
    NEKB_CUDA(cudaMemcpyAsync(bp->mask.p, mask.data(), sizeof(int32_t) * mask.size(),
                              cudaMemcpyHostToDevice, s));
  }

  // FP64 solver workspace (zeroed: the flexible beta reads Ap on the first iteration)
  const size_t vb = sizeof(double) * bp->Nfields * bp->offset;
  for (DeviceBuf* w : {&bp->p, &bp->z, &bp->Ap, &bp->Ax}) {
    NEKB_TRY(w->ensure(vb));
    NEKB_CUDA(cudaMemsetAsync(w->p, 0, vb, s));
  }
  NEKB_TRY(bp->invDiag.ensure(sizeof(double) * bp->offset));
  NEKB_TRY(bp->partials.ensure(sizeof(double) * 4 * 4096));
  NEKB_TRY(bp->counter.ensure(sizeof(unsigned) * 16));
  NEKB_CUDA(cudaMemsetAsync(bp->counter.p, 0, sizeof(unsigned) * 16, s));
  NEKB_TRY(bp->state.ensure(sizeof(PcgState)));
  NEKB_CUDA(cudaMallocHost(&bp->h_state, sizeof(PcgState)));
  NEKB_CUDA(cudaStreamSynchronize(s));
  return NEKB_OK;
}

// problem on the caller's mesh: ggeo (device, reference layout), global ids
// (host), mask list (host) and, optionally, the element vertices
static int bp_build_mesh(nekb_bp* bp, int N, int64_t E, int Nfields, const double* ggeo,
                         const int64_t* ids, int64_t Nmasked, const int32_t* maskIds,
                         const double* EX, const double* EY, const double* EZ,
                         cudaStream_t user_stream)
{
  bp->cfg = nekb_bp_config{};
  bp->cfg.N = N;
  bp->cfg.Nfields = Nfields;
  bp->N = N;
  bp->Nq = N + 1;
  bp->Np = bp->Nq * bp->Nq * bp->Nq;
  bp->Nfields = Nfields;
  bp->E = E;
  bp->Nlocal = E * bp->Np;
  bp->offset = bp->Nlocal;
  if (bp->Nlocal > INT32_MAX) return fail(NEKB_ERR_INVALID, "BP: %lld local nodes exceed 32-bit ids", (long long)bp->Nlocal);
  if (user_stream) {
    bp->stream = user_stream;
  } else {
    NEKB_CUDA(cudaStreamCreateWithFlags(&bp->stream, cudaStreamNonBlocking));
    bp->own_stream = true;
  }
  cudaStream_t s = bp->stream;
  NEKB_TRY(gll_nodes(N, bp->r1d, bp->w1d));
  const int Nq = bp->Nq;
  const int64_t Nl = bp->Nlocal;
  NEKB_TRY(bp->ggeo.ensure(sizeof(double) * 7 * Nl));
  NEKB_CUDA(cudaMemcpyAsync(bp->ggeo.p, ggeo, sizeof(double) * 7 * Nl, cudaMemcpyDefault, s));
  if (EX && EY && EZ) {
    for (auto pr : {std::make_pair(&bp->EX, EX), std::make_pair(&bp->EY, EY), std::make_pair(&bp->EZ, EZ)}) {
      NEKB_TRY(pr.first->ensure(sizeof(double) * 8 * E));
      NEKB_CUDA(cudaMemcpyAsync(pr.first->p, pr.second, sizeof(double) * 8 * E, cudaMemcpyDefault, s));
    }
    NEKB_TRY(bp->tri.ensure(sizeof(float) * 24 * E));
    NEKB_TRY(launch_trilinear_coeffs(E, bp->EX.as<double>(), bp->EY.as<double>(), bp->EZ.as<double>(),
                                     bp->tri.as<float>(), s));
  }
  std::vector<double> hD(Nq * Nq);
  deriv_matrix(Nq, bp->r1d, hD.data());
  std::vector<float> hDf(Nq * Nq);
  for (int t = 0; t < Nq * Nq; ++t) hDf[t] = (float)hD[t];
  NEKB_TRY(bp->D.ensure(sizeof(double) * Nq * Nq));
  NEKB_TRY(bp->Df.ensure(sizeof(float) * Nq * Nq));
  NEKB_CUDA(cudaMemcpyAsync(bp->D.p, hD.data(), sizeof(double) * Nq * Nq, cudaMemcpyHostToDevice, s));
  NEKB_CUDA(cudaMemcpyAsync(bp->Df.p, hDf.data(), sizeof(float) * Nq * Nq, cudaMemcpyHostToDevice, s));
  bp->ogs = new nekb_ogs();
  NEKB_TRY(nekb_ogs_build(bp->ogs, Nl, ids));
  bp->Nmasked = Nmasked;
  if (Nmasked > 0) {
    for (int64_t m = 0; m < Nmasked; ++m)
      if (maskIds[m] < 0 || maskIds[m] >= Nl) return fail(NEKB_ERR_INVALID, "BP: mask id %d out of range", maskIds[m]);
    NEKB_TRY(bp->mask.ensure(sizeof(int32_t) * Nmasked));
    NEKB_CUDA(cudaMemcpyAsync(bp->mask.p, maskIds, sizeof(int32_t) * Nmasked, cudaMemcpyHostToDevice, s));
  }
  const size_t vb = sizeof(double) * bp->Nfields * bp->offset;
  for (DeviceBuf* w : {&bp->p, &bp->z, &bp->Ap, &bp->Ax}) {
    NEKB_TRY(w->ensure(vb));
    NEKB_CUDA(cudaMemsetAsync(w->p, 0, vb, s));
  }
  NEKB_TRY(bp->invDiag.ensure(sizeof(double) * bp->offset));
  NEKB_TRY(bp->partials.ensure(sizeof(double) * 4 * 4096));
  NEKB_TRY(bp->counter.ensure(sizeof(unsigned) * 16));
  NEKB_CUDA(cudaMemsetAsync(bp->counter.p, 0, sizeof(unsigned) * 16, s));
  NEKB_TRY(bp->state.ensure(sizeof(PcgState)));
  NEKB_CUDA(cudaMallocHost(&bp->h_state, sizeof(PcgState)));
  NEKB_CUDA(cudaStreamSynchronize(s));
  return NEKB_OK;
}

}  // namespace nekb

nekb_bp* nekb_bp_create_mesh(int N, int64_t E, int Nfields, const double* ggeo, const int64_t* ids,
                             int64_t Nmasked, const int32_t* maskIds, const double* EX,
                             const double* EY, const double* EZ, void* stream, int* status)
{
  using namespace nekb;
  int st = NEKB_OK;
  nekb_bp* bp = nullptr;
  if (N < 1 || N + 1 > kMaxNq) {
    st = fail(NEKB_ERR_UNSUPPORTED, "BP: N=%d outside 1..%d", N, kMaxNq - 1);
  } else if (E < 1 || !ggeo || !ids || Nmasked < 0 || (Nmasked > 0 && !maskIds)) {
    st = fail(NEKB_ERR_INVALID, "BP: bad mesh arrays");
  } else if (Nfields != 1 && Nfields != 3) {
    st = fail(NEKB_ERR_INVALID, "BP: Nfields=%d (1 or 3)", Nfields);
  } else {
    bp = new nekb_bp();
    st = bp_build_mesh(bp, N, E, Nfields, ggeo, ids, Nmasked, maskIds, EX, EY, EZ,
                       static_cast<cudaStream_t>(stream));
    if (st != NEKB_OK) {
      nekb_bp_destroy(bp);
      bp = nullptr;
    }
  }
  if (status) *status = st;
  return bp;
}

void nekb_ogs_release(nekb_ogs* o)
{
  if (!o) return;
  cudaFree(o->d_chunks);
  cudaFree(o->d_pairs);
  cudaFree(o->d_quads);
  cudaFree(o->d_offsets);
  cudaFree(o->d_ids);
  cudaFree(o->d_invDegree);
  delete o;
}

nekb_bp* nekb_bp_create(const nekb_bp_config* cfg, void* stream, int* status)
{
  using namespace nekb;
  int st = NEKB_OK;
  nekb_bp* bp = nullptr;
  if (!cfg) {
    st = fail(NEKB_ERR_INVALID, "BP: config is NULL");
  } else if (cfg->N < 1 || cfg->N + 1 > kMaxNq) {
    st = fail(NEKB_ERR_UNSUPPORTED, "BP: N=%d outside 1..%d", cfg->N, kMaxNq - 1);
  } else if (cfg->nx < 1 || cfg->ny < 1 || cfg->nz < 1) {
    st = fail(NEKB_ERR_INVALID, "BP: box %dx%dx%d", cfg->nx, cfg->ny, cfg->nz);
  } else if (cfg->Nfields != 1 && cfg->Nfields != 3) {
    st = fail(NEKB_ERR_INVALID, "BP: Nfields=%d (1 or 3)", cfg->Nfields);
  } else if (cfg->periodic && (cfg->nx < 2 || cfg->ny < 2 || cfg->nz < 2)) {
    st = fail(NEKB_ERR_INVALID, "BP: periodic box needs at least 2 elements per direction");
  } else {
    bp = new nekb_bp();
    st = bp_build(bp, *cfg, static_cast<cudaStream_t>(stream));
    if (st != NEKB_OK) {
      nekb_bp_destroy(bp);
      bp = nullptr;
    }
  }
  if (status) *status = st;
  return bp;
}

void nekb_bp_destroy(nekb_bp* bp)
{
  if (!bp) return;
  for (auto& kv : bp->graphs) cudaGraphExecDestroy(kv.second);
  bp->graphs.clear();
  if (bp->stream) cudaStreamSynchronize(bp->stream);
  nekb_ogs_release(bp->ogs);
  if (bp->h_state) cudaFreeHost(bp->h_state);
  cudaStream_t s = bp->own_stream ? bp->stream : nullptr;
  delete bp;  // frees the device buffers
  if (s) cudaStreamDestroy(s);  // a caller's stream is left alone
}
