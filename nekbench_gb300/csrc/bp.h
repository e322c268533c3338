// Benchmark-problem state (mesh, geometry, gather-scatter, solver workspace):
// the data the reference keeps in mesh_t and BP_t (nekBone/BP.hpp:47-153).
#pragma once

#include "internal.h"

#include <map>
#include <tuple>

namespace nekb {

// operator Aq = mask(gs(axhelm(q))) in one precision
struct OpView {
  int Nq = 0;
  int flags = 0;       // NEKB_AX_BK / NEKB_AX_N3
  int precision = 0;   // NEKB_FP64, NEKB_FP32, NEKB_BF16, NEKB_FP32_TRILINEAR
  int Nfields = 1;
  int64_t E = 0;
  int64_t offset = 0;  // field stride (= E*Np)
  const void* ggeo = nullptr;
  const void* D = nullptr;
  const void* lambda = nullptr;
  const nekb_ogs* ogs = nullptr;
  const int32_t* mask = nullptr;
  int64_t Nmasked = 0;
  float r1d[kMaxNq] = {};
  float w1d[kMaxNq] = {};
};

// Aq = mask(gs(axhelm(q))); with dot_partials, the operator kernel also leaves
// per-block sums of q . axhelm(q) (before assembly) and their count
int apply_op(const OpView& op, const void* q, void* Aq, const int* skip, cudaStream_t s,
             double* dot_partials = nullptr, int* dot_count = nullptr);

// longest window of truncated flexible CG, FCG(m)
constexpr int kFcgMax = 8;

// device state of one PCG run; updated by the last block of each reduction
struct PcgState {
  double rdotz1, rdotz2, rdotr, rdotr0, TOL, alpha, beta, pAp, tol2, zdotAp;
  int iter, done, result, status, maxit, flexible, fixed, pad;
  // FCG(m): z . A p_j of the current z and p_j . A p_j for the kept
  // directions (ring slots), the window m, the directions kept and the slot
  // the next direction goes to
  double fcg_zap[kFcgMax], fcg_pap[kFcgMax];
  int fcg_m, fcg_count, fcg_head, fcg_pad;
};

struct DeviceBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t b);
  ~DeviceBuf();
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace nekb

struct nekb_bp {
  nekb_bp_config cfg{};
  int N = 0, Nq = 0, Np = 0, Nfields = 1;
  int64_t E = 0, Nlocal = 0, offset = 0, Nmasked = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  double r1d[nekb::kMaxNq] = {}, w1d[nekb::kMaxNq] = {};
  nekb_ogs* ogs = nullptr;
  // geometry and basis (device)
  nekb::DeviceBuf EX, EY, EZ, ggeo, D, Df, tri, mask, xyz;
  nekb::DeviceBuf ggeo_f, ggeo_bf, invdeg_f;
  // FP64 workspace: p, z, Ap, Ax, invDiag, b, r (outer residual)
  nekb::DeviceBuf p, z, Ap, Ax, invDiag, b, rr;
  // FP32 workspace of the inner solver
  nekb::DeviceBuf r32, x32, p32, z32, Ap32, invDiag32, lam32;
  // FCG(m) directions p_j and A p_j (kFcgMax slots of Nfields*offset floats each)
  nekb::DeviceBuf fcgP, fcgAP;
  // per-block p . A p sums of the FP32 operator (one per operator block) + count
  nekb::DeviceBuf axdot;
  // reduction scratch and solver state
  nekb::DeviceBuf partials, counter, state;
  nekb::PcgState* h_state = nullptr;  // pinned mirror
  // CUDA graphs of one chunk of PCG iterations, keyed by their arguments and,
  // with the learned preconditioner, by the network, its weights' address and
  // the inference kernel it runs (a graph replays the launches it captured)
  std::map<std::tuple<int, int, int, const void*, const void*, const void*, int, const void*, const void*, int>,
           cudaGraphExec_t>
      graphs;
  void* net = nullptr;  // learned preconditioner in use (nekb_net*)
};

namespace nekb {
// BPZeroMean (nekBone/solve.cpp:115-134) on the problem's stream, asynchronous
int bp_zero_mean(nekb_bp* bp, double* q);
}  // namespace nekb
