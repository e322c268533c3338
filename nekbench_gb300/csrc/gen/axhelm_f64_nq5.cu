// axhelm instantiation: precision NEKB_FP64, Nq=5.
#include "../axhelm_impl.cuh"

namespace nekb {
int launch_axhelm_f64_nq5(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax::run_flags<5, NEKB_FP64>(flags, a, s);
}
}  // namespace nekb
