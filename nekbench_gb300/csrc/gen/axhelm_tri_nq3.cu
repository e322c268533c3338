// axhelm instantiation: precision NEKB_FP32_TRILINEAR, Nq=3.
#include "../axhelm_impl.cuh"

namespace nekb {
int launch_axhelm_tri_nq3(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax::run_flags<3, NEKB_FP32_TRILINEAR>(flags, a, s);
}
}  // namespace nekb
