// Instantiations of the adv operator kernel (adv_impl.cuh) for (Nq, cubNq) = (9, 14), (10, 15).
#include "adv_impl.cuh"

namespace nekb {
namespace adv {
template int launch<9, 14>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<10, 15>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
}  // namespace adv
}  // namespace nekb
