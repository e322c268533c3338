// C-linkage shim over the reference's own CPU axhelm sources (test infrastructure).
//
// oracle/Makefile compiles this file together with, straight from the
// nekBench source tree:
//   axhelm/axhelmReference.cpp      (axhelmReference, :91)
//   axhelm/kernel/CPU/axhelm.c      (axhelm_v0 :27, axhelm_n3_v0 :113,
//                                    axhelm_bk_v0 :229, axhelm_bk_n3_v0 :307)
//   nekBone/kernel/CPU/weightedInnerProduct.c (weightedInnerProductUpdate :64)
// with -Ddfloat=double -Ddlong=int -Dp_Nq=<Nq> -include core/params.h, and
// exposes them with plain C names so the tests can call them through ctypes.
// Nothing here is part of the library.

void axhelmReference(int Nq, const int numElements, dfloat lambda, const dfloat* ggeo,
                     const dfloat* D, const dfloat* solIn, dfloat* solOut);

extern "C" {
void axhelm_v0(const dlong&, const dlong&, const dfloat*, const dfloat*, const dfloat*,
               const dfloat*, dfloat*);
void axhelm_n3_v0(const dlong&, const dlong&, const dfloat*, const dfloat*, const dfloat*,
                  const dfloat*, dfloat*);
void axhelm_bk_v0(const dlong&, const dlong&, const dfloat*, const dfloat*, const dfloat*,
                  const dfloat*, dfloat*);
void axhelm_bk_n3_v0(const dlong&, const dlong&, const dfloat*, const dfloat*, const dfloat*,
                     const dfloat*, dfloat*);
void weightedInnerProductUpdate(const dlong&, const dlong&, const dlong&, const dfloat*,
                                const dfloat*, const dfloat*, dfloat*);

int nekref_nq(void) { return p_Nq; }

void nekref_axhelm_reference(int Nq, int numElements, double lambda, const double* ggeo,
                             const double* D, const double* q, double* Aq)
{
  axhelmReference(Nq, numElements, lambda, ggeo, D, q, Aq);
}

// variant: bit0 = BK, bit1 = n3 (same meaning as the library's flags)
int nekref_axhelm_cpu(int variant, int Nelements, int offset, const double* ggeo, const double* D,
                      const double* lambda, const double* q, double* Aq)
{
  const dlong E = Nelements, off = offset;
  switch (variant & 3) {
    case 0: axhelm_v0(E, off, ggeo, D, lambda, q, Aq); return 0;
    case 1: axhelm_bk_v0(E, off, ggeo, D, lambda, q, Aq); return 0;
    case 2: axhelm_n3_v0(E, off, ggeo, D, lambda, q, Aq); return 0;
    case 3: axhelm_bk_n3_v0(E, off, ggeo, D, lambda, q, Aq); return 0;
  }
  return -1;
}

void nekref_weighted_inner_product_update(int N, int offset, const double* w, const double* a,
                                          const double* b, double* wab)
{
  const dlong n = N, off = offset, nb = 1;
  weightedInnerProductUpdate(n, off, nb, w, a, b, wab);
}
}
