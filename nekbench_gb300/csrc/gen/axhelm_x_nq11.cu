// axhelm instantiation: FP64 arrays, double-float arithmetic, Nq=11.
#include "../axhelm_x.cuh"

namespace nekb {
int launch_axhelm_x_nq11(int flags, const AxArgs& a, cudaStream_t s)
{
  return axx::run_flags<11>(flags, a, s);
}
}  // namespace nekb
