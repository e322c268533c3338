// axhelm instantiation: FP64 arrays, double-float arithmetic, Nq=9.
#include "../axhelm_x.cuh"

namespace nekb {
int launch_axhelm_x_nq9(int flags, const AxArgs& a, cudaStream_t s)
{
  return axx::run_flags<9>(flags, a, s);
}
}  // namespace nekb
