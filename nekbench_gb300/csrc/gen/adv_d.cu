// Instantiations of the adv operator kernel (adv_impl.cuh) for (Nq, cubNq) = (11, 11), (12, 12).
#include "adv_impl.cuh"

namespace nekb {
namespace adv {
template int launch<11, 11>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<12, 12>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
}  // namespace adv
}  // namespace nekb
