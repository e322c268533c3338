// C entry of the adv benchmark's advection operator (advCubatureHex3D_v0,
// adv/kernel/VOLTA/adv.okl:27-261): argument checks and the dispatch to the
// kernel built for the (Nq, cubNq) pair; the kernel is adv_impl.cuh, its
// instantiations are csrc/gen/adv_*.cu.
#include "internal.h"

namespace nekb {
namespace adv {
template <int NQ, int CQ>
int launch(bool split, int64_t E, const double* vgeo, const double* cubvgeo, const double* cubD,
           const double* cubInterpT, int64_t offset, const double* U, double* NU, cudaStream_t s);
}  // namespace adv

namespace {

using Launcher = int (*)(bool, int64_t, const double*, const double*, const double*, const double*, int64_t,
                         const double*, double*, cudaStream_t);

// cubNq = Nq (Nq = 2..12) and the 3/2 rule cubNq = ceil(3 Nq / 2) (Nq = 2..10)
Launcher find_launcher(int Nq, int cubNq)
{
#define NEKB_ADV(nq, cq) \
  if (Nq == nq && cubNq == cq) return adv::launch<nq, cq>;
  NEKB_ADV(2, 2) NEKB_ADV(3, 3) NEKB_ADV(4, 4) NEKB_ADV(5, 5) NEKB_ADV(6, 6) NEKB_ADV(7, 7)
  NEKB_ADV(8, 8) NEKB_ADV(9, 9) NEKB_ADV(10, 10) NEKB_ADV(11, 11) NEKB_ADV(12, 12)
  NEKB_ADV(2, 3) NEKB_ADV(3, 5) NEKB_ADV(4, 6) NEKB_ADV(5, 8) NEKB_ADV(6, 9) NEKB_ADV(7, 11)
  NEKB_ADV(8, 12) NEKB_ADV(9, 14) NEKB_ADV(10, 15)
#undef NEKB_ADV
  return nullptr;
}

}  // namespace
}  // namespace nekb

extern "C" int nekb_adv_cubature(int Nq, int cubNq, int precision, int64_t Nelements,
                                 const double* vgeo,
                                 const double* cubvgeo, const double* cubD, const double* cubInterpT,
                                 int64_t offset, const double* U, double* NU, void* stream)
{
  using namespace nekb;
  const auto fn = find_launcher(Nq, cubNq);
  if (!fn)
    return fail(NEKB_ERR_UNSUPPORTED,
                "adv: Nq=%d cubNq=%d not built (cubNq = Nq for Nq 2..12, cubNq = ceil(3 Nq/2) "
                "for Nq 2..10)", Nq, cubNq);
  if (precision != NEKB_FP64 && precision != NEKB_FP64_SPLIT)
    return fail(NEKB_ERR_UNSUPPORTED, "adv: precision %d (NEKB_FP64 or NEKB_FP64_SPLIT)", precision);
  const int64_t Np = (int64_t)Nq * Nq * Nq;
  if (Nelements < 0 || Nelements > INT32_MAX || offset < Nelements * Np)
    return fail(NEKB_ERR_INVALID, "adv: Nelements=%lld offset=%lld (offset >= Nelements*Np)",
                (long long)Nelements, (long long)offset);
  if (Nelements == 0) return NEKB_OK;
  if (!vgeo || !cubvgeo || !cubD || !cubInterpT || !U || !NU)
    return fail(NEKB_ERR_INVALID, "adv: NULL argument");
  return fn(precision == NEKB_FP64_SPLIT, Nelements, vgeo, cubvgeo, cubD, cubInterpT, offset, U, NU,
            static_cast<cudaStream_t>(stream));
}
