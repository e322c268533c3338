// Learned element preconditioner: internal interface used by the PCG driver.
#pragma once

#include "bp.h"

#include <cuda_bf16.h>

namespace nekb {

// z = Jacobi(r) + mask(gs(w * h * s_e * net(h * r_e / s_e))), h = sqrt(invDiag),
// s_e = RMS of h * r over element e.
// Runs on stream s; returns at once on the device when *skip != 0.
int net_precondition(nekb_bp* bp, nekb_net* net, const float* r, float* z, const float* invDiag,
                     const float* w, const int* skip, cudaStream_t s);

// The flexible CG's update folded into the tcgen05 network kernel: before an
// element is evaluated, r_e -= alpha Ap_e (written back to r) and
// x_e += alpha p_e, with alpha = (float) *alpha read on the device -- the
// arithmetic of the separate update pass.
struct NetUpdate {
  const double* alpha;
  const float* Ap;
  const float* p;
  float* x;
};
// whether net_precondition_update can fold the update (the tcgen05 kernel runs)
bool net_takes_update(const nekb_net* net);
// the update above, then net_precondition on the updated r
int net_precondition_update(nekb_bp* bp, nekb_net* net, const NetUpdate& up, float* r, float* z,
                            const float* invDiag, const float* w, const int* skip, cudaStream_t s);

// what a captured PCG graph bakes in from the network: its order, channels,
// the inference kernel that runs (the resolved mode) and its weights' address
struct NetSignature {
  const void* net;
  const void* weights;
  int shape_mode;  // (Nq * 100 + C) * 8 + resolved mode
};
NetSignature net_signature(const nekb_net* net);

// inference mode bits: normalise by the element RMS of sqrt(invDiag) r; add
// w invDiag r to the output
constexpr int kNetNormalize = 1, kNetAddJacobi = 2;

// tensor-core inference, Nq=8, 16 channels: tcgen05 MMAs with TMEM
// accumulators (nn_tc5.cu) and warp-level mma.sync (nn_tc.cu)
bool net_tc_supported(int Nq, int C);
int net_infer_tc5(const __nv_bfloat16* Wbf, int64_t Etot, int64_t Efield, const float* r,
                  const float* w, const float* invDiag, float* out, int normalize, const int* skip,
                  cudaStream_t s, const NetUpdate* up = nullptr);
int net_infer_tc(const __nv_bfloat16* Wbf, int64_t Etot, int64_t Efield, const float* r,
                 const float* w, const float* invDiag, float* out, int normalize, const int* skip,
                 cudaStream_t s);
// NEKB_OK, or an error (and the flags cleared) when a tensor-core launch gave
// up waiting for its input copies or its MMAs since the last call
int net_tc_copy_timeout();
// sets the timeout flags from the host, as the kernels do when a wait runs out
// (for tests of the error path; no device wait runs out)
int net_tc_raise_copy_timeout();
int net_tc5_take_timeout(int* flag);
int net_tc5_raise_timeout();

}  // namespace nekb
