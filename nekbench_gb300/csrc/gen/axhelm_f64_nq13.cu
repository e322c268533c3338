// axhelm instantiation: precision NEKB_FP64, Nq=13 (even-odd contractions).
#include "../axhelm_eo.cuh"

namespace nekb {
int launch_axhelm_f64_nq13(int flags, const AxArgs& a, cudaStream_t s)
{
  return ax_eo::run_flags<13>(flags, a, s);
}
}  // namespace nekb
