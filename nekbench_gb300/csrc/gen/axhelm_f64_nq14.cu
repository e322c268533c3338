// axhelm instantiation: precision NEKB_FP64, Nq=14 (even-odd contractions).
#include "../axhelm_eo.cuh"

namespace nekb {
int launch_axhelm_f64_nq14(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax_eo::run_flags<14>(flags, a, s);
}
}  // namespace nekb
