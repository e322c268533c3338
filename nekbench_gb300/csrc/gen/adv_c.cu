// Instantiations of the adv operator kernel (adv_impl.cuh) for (Nq, cubNq) = (10, 10), (7, 11), (8, 12).
#include "adv_impl.cuh"

namespace nekb {
namespace adv {
template int launch<10, 10>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<7, 11>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<8, 12>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
}  // namespace adv
}  // namespace nekb
