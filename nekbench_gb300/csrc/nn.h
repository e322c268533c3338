// Learned element preconditioner: internal interface used by the PCG driver.
#pragma once

#include "bp.h"

namespace nekb {

// z = Jacobi(r) + mask(gs(w * s_e * net(r_e / s_e))), s_e = RMS of r over element e.
// Runs on stream s; returns at once on the device when *skip != 0.
int net_precondition(nekb_bp* bp, nekb_net* net, const float* r, float* z, const float* invDiag,
                     const float* w, const int* skip, cudaStream_t s);

}  // namespace nekb
