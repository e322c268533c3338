// axhelm instantiation: FP64 arrays, double-float arithmetic, Nq=12.
#include "../axhelm_x.cuh"

namespace nekb {
int launch_axhelm_x_nq12(int flags, const AxArgs& a, cudaStream_t s)
{
  return axx::run_flags<12>(flags, a, s);
}
}  // namespace nekb
