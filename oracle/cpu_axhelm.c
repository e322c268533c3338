/* CPU baseline of the benchmark: the reference's CPU axhelm timed beside the
 * GPU (test and benchmark infrastructure; never linked by the library).
 *
 * The reference compiles axhelm/kernel/CPU/axhelm.c once per order with p_Nq
 * and p_Np defined (axhelm/kernelHelper.cpp:18-33) and OCCA's default flags,
 * "-O3" (3rdParty/occa/src/modes/serial/device.cpp:47), under which the
 * compiler may fuse multiply-adds.  This file restates those loop nests
 * (cpu_axhelm_body.h) with the order fixed at compile time, one copy per order
 * 2..14, built the same way (oracle/Makefile: -O3, GNU C, OpenMP over
 * elements).  Its results agree with the bit-identical restatement in
 * nekb_oracle.c to rounding (about 1e-15 relative where fused multiply-adds
 * are used); that file stays the checker, this one is the timed baseline. */
#include <stdint.h>

#define CB_CAT_(a, b) a##b
#define CB_CAT(a, b) CB_CAT_(a, b)

#define NQ 2
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 3
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 4
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 5
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 6
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 7
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 8
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 9
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 10
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 11
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 12
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 13
#include "cpu_axhelm_body.h"
#undef NQ
#define NQ 14
#include "cpu_axhelm_body.h"
#undef NQ

/* single-field axhelm (bk: Poisson, lambda unused) on E elements; returns 0,
 * or -1 for an order outside 2..14 */
int nekbc_axhelm(int Nq, int bk, int64_t E, int64_t offset, const double* ggeo, const double* D,
                 const double* lambda, const double* q, double* Aq)
{
  switch (Nq) {
    case 2: cb_axhelm_nq2(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 3: cb_axhelm_nq3(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 4: cb_axhelm_nq4(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 5: cb_axhelm_nq5(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 6: cb_axhelm_nq6(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 7: cb_axhelm_nq7(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 8: cb_axhelm_nq8(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 9: cb_axhelm_nq9(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 10: cb_axhelm_nq10(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 11: cb_axhelm_nq11(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 12: cb_axhelm_nq12(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 13: cb_axhelm_nq13(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
    case 14: cb_axhelm_nq14(bk, E, offset, ggeo, D, lambda, q, Aq); return 0;
  }
  return -1;
}
