// axhelm instantiation: precision NEKB_BF16, Nq=6.
#include "../axhelm_impl.cuh"

namespace nekb {
int launch_axhelm_bf16_nq6(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax::run_flags<6, NEKB_BF16>(flags, a, s);
}
}  // namespace nekb
