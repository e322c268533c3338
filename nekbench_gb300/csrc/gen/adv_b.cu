// Instantiations of the adv operator kernel (adv_impl.cuh) for (Nq, cubNq) = (8, 8), (9, 9), (5, 8), (6, 9).
#include "adv_impl.cuh"

namespace nekb {
namespace adv {
template int launch<8, 8>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<9, 9>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<5, 8>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<6, 9>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
}  // namespace adv
}  // namespace nekb
