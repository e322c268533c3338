// axhelm instantiation: FP64 arrays, double-float arithmetic, Nq=5.
#include "../axhelm_x.cuh"

namespace nekb {
int launch_axhelm_x_nq5(int flags, const AxArgs& a, cudaStream_t s)
{
  return axx::run_flags<5>(flags, a, s);
}
}  // namespace nekb
