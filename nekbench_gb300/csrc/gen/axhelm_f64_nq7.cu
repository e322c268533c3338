// axhelm instantiation: precision NEKB_FP64, Nq=7 (even-odd contractions).
#include "../axhelm_eo.cuh"

namespace nekb {
int launch_axhelm_f64_nq7(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax_eo::run_flags<7>(flags, a, s);
}
}  // namespace nekb
