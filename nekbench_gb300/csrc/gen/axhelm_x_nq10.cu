// axhelm instantiation: FP64 arrays, double-float arithmetic, Nq=10.
#include "../axhelm_x.cuh"

namespace nekb {
int launch_axhelm_x_nq10(int flags, const AxArgs& a, cudaStream_t s)
{
  return axx::run_flags<10>(flags, a, s);
}
}  // namespace nekb
