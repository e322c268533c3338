// axhelm instantiation: precision NEKB_FP32, Nq=11.
#include "../axhelm_impl.cuh"

namespace nekb {
int launch_axhelm_f32_nq11(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax::run_flags<11, NEKB_FP32>(flags, a, s);
}
}  // namespace nekb
