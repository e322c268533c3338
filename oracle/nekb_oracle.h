/*
 * CPU oracle for the nekBench spectral-element hot path (test infrastructure).
 *
 * This file and nekb_oracle.c restate, in plain C, the reference algorithms
 * the GPU library must reproduce.  They are the CHECKER, never the product:
 * only the test-suite, the smoke check and the CPU-baseline leg of the
 * benchmark may call them.  Every function cites the reference file:line it
 * restates (paths relative to the nekBench source tree).
 *
 * Pinning: the axhelm restatement is checked against the reference's own
 * axhelm/axhelmReference.cpp and axhelm/kernel/CPU/axhelm.c (compiled from the
 * reference sources into oracle/_ref by oracle/Makefile) and against golden
 * vectors committed under tests/golden/.  The gather-scatter restatement is
 * checked with the reference's own known-answer test (gs/main.cpp:136-193).
 */
#ifndef NEKB_ORACLE_H
#define NEKB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* axhelm variant flags (same bit meaning as the library's NEKB_AX_* flags) */
#define NEKBO_AX_BK      1  /* Poisson mode: lambda0 = 1, no lambda1 term, no lambda reads */
#define NEKBO_AX_N3      2  /* three fields sharing ggeo/lambda, stride = offset          */
#define NEKBO_AX_PARTIAL 4  /* element list                                              */

/* ---- counter-based random numbers shared bit-for-bit with the library ---- */
uint64_t nekbo_hash(uint64_t seed, uint64_t stream, uint64_t i);
double   nekbo_uniform(uint64_t seed, uint64_t stream, uint64_t i);
void     nekbo_fill_uniform(double* v, int64_t n, uint64_t seed, uint64_t stream,
                            double lo, double hi);

/* ---- 1D basis (core/meshBasis.cpp:46 meshJacobiGQ, :140 meshJacobiGL, :775 meshDmatrix1D) ---- */
int  nekbo_gll(int N, double* x, double* w);     /* N+1 Gauss-Lobatto-Legendre nodes/weights */
int  nekbo_gauss(int N, double* x, double* w);   /* N+1 Gauss-Legendre nodes/weights          */
void nekbo_dmatrix(int Nq, const double* x, double* D); /* D[i*Nq+m] = l_m'(x_i)              */

/* ---- box mesh (core/meshSetup.cpp:2265 meshSetupBoxHex3D, :2156 meshPhysicalNodesHex3D) ---- */
void    nekbo_box_vertices(int nx, int ny, int nz, double perturb, uint64_t seed, int periodic,
                           double box_min, double box_max, double* EX, double* EY, double* EZ);
void    nekbo_box_ids(int N, int nx, int ny, int nz, int periodic, int dirichlet, int64_t* ids);
int64_t nekbo_box_mask(int N, int nx, int ny, int nz, int32_t* maskIds /* nullable: count only */);
void    nekbo_physical_nodes(int N, int64_t E, const double* r1d, const double* EX,
                             const double* EY, const double* EZ, double* x, double* y, double* z);
void    nekbo_geometric_factors(int N, int64_t E, const double* w1d, const double* D,
                                const double* x, const double* y, const double* z, double* ggeo);

/* ---- axhelm (axhelm/kernel/CPU/axhelm.c:27,113,229,307; axhelm/axhelmReference.cpp:91) ---- */
void nekbo_axhelm(int Nq, int64_t Nelements, int64_t offset, int flags, const int32_t* elementList,
                  const double* ggeo, const double* D, const double* lambda,
                  const double* q, double* Aq);
/* same operator, loops parallelised over elements with OpenMP: the CPU baseline */
void nekbo_axhelm_omp(int Nq, int64_t Nelements, int64_t offset, int flags,
                      const double* ggeo, const double* D, const double* lambda,
                      const double* q, double* Aq);
int  nekbo_omp_threads(void);

/* ---- ogs local gather-scatter (3rdParty/ogs/src/ogsSetup.cpp:137-212, 325-352;
 *      3rdParty/ogs/okl/gatherScatterMany.okl:58) ---- */
int64_t nekbo_ogs_setup(int64_t N, const int64_t* ids, int32_t* offsets /* N+1 */,
                        int32_t* gatherIds /* N */, double* invDegree /* N */);
void    nekbo_gs_many_add(int64_t Ngather, const int32_t* offsets, const int32_t* gatherIds,
                          int k, int64_t stride, double* q);
void    nekbo_mask(int64_t Nmasked, const int32_t* maskIds, double* q); /* utils.okl:127 */

/* ---- Jacobi diagonal (nekBone/kernel/updateJacobi.okl:27-108) ---- */
void nekbo_update_jacobi(int Nq, int64_t Nelements, int64_t offset, const int32_t* mapB,
                         const double* ggeo, const double* D, const double* lambda, double* diag);

/* ---- nekBone PCG (nekBone/solve.cpp:44-113) ---- */
typedef struct {
  int Nq;
  int64_t Nelements;
  int Nfields;
  int64_t offset;          /* field offset (= Nelements*Np on one rank)           */
  int bk;                  /* BK operator (lambda0=1, lambda1=0)                   */
  const double* ggeo;
  const double* D;
  const double* lambda;    /* 2*offset: lambda0 then lambda1                      */
  int64_t Ngather;
  const int32_t* gatherOffsets;
  const int32_t* gatherIds;
  const double* invDegree;
  int64_t Nmasked;
  const int32_t* maskIds;
} nekbo_bp;

/* precond: 0 = COPY, 1 = JACOBI.  Returns the iteration count as BPPCG does
 * (iter-1 at exit).  rdotr_hist (nullable, maxit+1 entries) gets rdotr per iteration. */
int nekbo_pcg(const nekbo_bp* bp, double* r, double* x, double tol, int maxit, int precond,
              int flexible, int fixed_iterations, double* rdotr_hist);
/* BPZeroMean (nekBone/solve.cpp:115-134): q -= (sum of the Nloc local values
 * of every field) / (Nloc*Nfields), over all Nfields*offset entries.  The sum
 * runs in index order (the reference sums 256-wide block partials). */
void nekbo_zero_mean(int64_t Nloc, int Nfields, int64_t offset, double* q);
/* BPPCG on all host threads (OpenMP loops and reductions): the CPU timing
 * baseline of the PCG, not a parity reference.  *setup_s (nullable) receives
 * the time of the initial residual and the Jacobi set-up. */
/* operator of the CPU baseline build (cpu_axhelm.c nekbc_axhelm): Nq, bk, E,
 * offset, ggeo, D, lambda, q, Aq; returns 0 when it handled the call */
typedef int (*nekbo_cpu_axhelm_fn)(int, int, int64_t, int64_t, const double*, const double*,
                                   const double*, const double*, double*);
void nekbo_set_cpu_axhelm(nekbo_cpu_axhelm_fn fn);
int nekbo_pcg_omp(const nekbo_bp* bp, double* r, double* x, double tol, int maxit, int precond,
                  int fixed_iterations, double* setup_s);
/* operator used by the PCG: Aq = mask(gs(axhelm(q))) */
void nekbo_bp_apply(const nekbo_bp* bp, const double* q, double* Aq);
double nekbo_wdot(int64_t N, int Nfields, int64_t offset, const double* w, const double* a,
                  const double* b);

/* ---- learned element preconditioner: 3D convolution network on Nq^3 element nodes ----
 * layer l: out[co][n] = sum_ci sum_tap W[l][co][ci][tap] * in[ci][n+tap] (zero padding),
 * followed by GELU (tanh form) on every layer but the last.  Channels: 1 -> C -> ... -> 1. */
void nekbo_conv3d_forward(int Nq, int64_t Nelem, int Cin, int Cout, const float* W /* Cout*Cin*27 */,
                          const float* in /* Nelem*Cin*Nq^3 */, float* out /* Nelem*Cout*Nq^3 */);
void nekbo_conv3d_backward(int Nq, int64_t Nelem, int Cin, int Cout, const float* W,
                           const float* in, const float* gout, float* gin /* nullable */,
                           float* gW /* Cout*Cin*27, accumulated (+=) */);
void nekbo_gelu_forward(int64_t n, const float* x, float* y);
void nekbo_gelu_backward(int64_t n, const float* x, const float* gy, float* gx);

/* ---- dot benchmark (dot/kernel/VOLTA/dot.okl) ----
 * Per-block partials wxy[b] of blockSize consecutive nodes, reduced in the
 * kernels' tree: variant 0 weightedInnerProduct2_v0 (dot.okl:27-65), 1
 * weightedInnerProduct2_v1 (dot.okl:114-169, its lockstep tree), 2
 * weightedBlockInnerProduct2 (dot.okl:67-111, Nfields triple products per
 * node).  Returns the number of blocks written, or -1 on bad arguments.
 * Variants 0 and 2 are pinned bit for bit to the reference's OKL kernels run
 * with OCCA's Serial semantics (tests/golden/okl_serial.npz); variant 1 only
 * computes the right sum in lockstep, so it is checked by its total. */
int64_t nekbo_dot_partials(int variant, int64_t N, int Nfields, int64_t offset, int blockSize,
                           const double* w, const double* x, const double* y, double* wxy);

/* ---- adv benchmark: advCubatureHex3D_v0 (adv/kernel/VOLTA/adv.okl:27-261) ----
 * NU_f = IJW . (I^T x I^T x I^T)[Uhat dUc_f/dr + Vhat dUc_f/ds + What dUc_f/dt],
 * Uc = (I x I x I) U, I(i <- a) = cubInterpT[a*cubNq + i]; metric slots of
 * core/params.h:2-13 (12 per node).  The t-projected slice is cubNq x cubNq
 * (the reference's s_U is Nq x Nq but indexed up to cubNq x cubNq,
 * adv.okl:203-231; the two agree for cubNq = Nq).  For cubNq = Nq pinned bit
 * for bit to the reference's OKL kernel run with OCCA's Serial semantics
 * (tests/golden/okl_serial.npz); for cubNq > Nq, where the reference's
 * kernel runs past s_U, checked against exact polynomial answers. */
void nekbo_adv_cubature(int Nq, int cubNq, int64_t Nelements, const double* vgeo,
                        const double* cubvgeo, const double* cubD, const double* cubInterpT,
                        int64_t offset, const double* U, double* NU);

#ifdef __cplusplus
}
#endif
#endif
