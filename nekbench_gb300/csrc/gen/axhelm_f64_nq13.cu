// axhelm instantiation: precision NEKB_FP64, Nq=13 (the largest orders are
// built for FP64 only).
#include "../axhelm_impl.cuh"

namespace nekb {
int launch_axhelm_f64_nq13(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax::run_flags<13, NEKB_FP64>(flags, a, s);
}
}  // namespace nekb
