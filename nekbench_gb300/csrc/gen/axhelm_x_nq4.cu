// axhelm instantiation: FP64 arrays, double-float arithmetic, Nq=4.
#include "../axhelm_x.cuh"

namespace nekb {
int launch_axhelm_x_nq4(int flags, const AxArgs& a, cudaStream_t s)
{
  return axx::run_flags<4>(flags, a, s);
}
}  // namespace nekb
