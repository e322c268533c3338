// axhelm instantiation: FP64 arrays, double-float arithmetic, Nq=7.
#include "../axhelm_x.cuh"

namespace nekb {
int launch_axhelm_x_nq7(int flags, const AxArgs& a, cudaStream_t s)
{
  return axx::run_flags<7>(flags, a, s);
}
}  // namespace nekb
