// axhelm instantiation: FP64 arrays, double-float arithmetic, Nq=3.
#include "../axhelm_x.cuh"

namespace nekb {
int launch_axhelm_x_nq3(int flags, const AxArgs& a, cudaStream_t s)
{
  return axx::run_flags<3>(flags, a, s);
}
}  // namespace nekb
