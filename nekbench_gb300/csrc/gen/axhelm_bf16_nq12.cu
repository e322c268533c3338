// axhelm instantiation: precision NEKB_BF16, Nq=12.
#include "../axhelm_impl.cuh"

namespace nekb {
int launch_axhelm_bf16_nq12(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax::run_flags<12, NEKB_BF16>(flags, a, s);
}
}  // namespace nekb
