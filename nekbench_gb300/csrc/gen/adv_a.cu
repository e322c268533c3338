// Instantiations of the adv operator kernel (adv_impl.cuh) for (Nq, cubNq) = (2, 2), (3, 3), (4, 4), (5, 5), (6, 6), (7, 7), (2, 3), (3, 5), (4, 6).
#include "adv_impl.cuh"

namespace nekb {
namespace adv {
template int launch<2, 2>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<3, 3>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<4, 4>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<5, 5>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<6, 6>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<7, 7>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<2, 3>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<3, 5>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
template int launch<4, 6>(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                            const double*, double*, cudaStream_t);
}  // namespace adv
}  // namespace nekb
