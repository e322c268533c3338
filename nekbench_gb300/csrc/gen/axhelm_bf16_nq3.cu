// axhelm instantiation: precision NEKB_BF16, Nq=3.
#include "../axhelm_impl.cuh"

namespace nekb {
int launch_axhelm_bf16_nq3(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax::run_flags<3, NEKB_BF16>(flags, a, s);
}
}  // namespace nekb
