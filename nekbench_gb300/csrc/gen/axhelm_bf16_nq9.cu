// axhelm instantiation: precision NEKB_BF16, Nq=9.
#include "../axhelm_impl.cuh"

namespace nekb {
int launch_axhelm_bf16_nq9(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax::run_flags<9, NEKB_BF16>(flags, a, s);
}
}  // namespace nekb
