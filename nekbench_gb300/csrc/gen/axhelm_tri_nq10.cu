// axhelm instantiation: precision NEKB_FP32_TRILINEAR, Nq=10.
#include "../axhelm_impl.cuh"

namespace nekb {
int launch_axhelm_tri_nq10(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax::run_flags<10, NEKB_FP32_TRILINEAR>(flags, a, s);
}
}  // namespace nekb
