// axhelm instantiation: precision NEKB_FP32, Nq=7.
#include "../axhelm_impl.cuh"

namespace nekb {
int launch_axhelm_f32_nq7(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax::run_flags<7, NEKB_FP32>(flags, a, s);
}
}  // namespace nekb
