/*
 * nekb -- GB300-native (sm_103a) spectral-element hot path of nekBench.
 *
 * Plain C ABI: device pointers and sizes, no C++ or framework types.  Every
 * entry point returns NEKB_OK (0) or a negative NEKB_ERR_* status; the text of
 * the last error on the calling thread is available from nekb_last_error().
 * Nothing here calls exit() or aborts.  Streams are passed as void* holding a
 * cudaStream_t (NULL = the legacy default stream).
 *
 * Memory layouts follow the reference exactly (paths relative to the nekBench
 * source tree):
 *   ggeo    [e*7*Np + slot*Np + n], slots GWJ,G00,G01,G02,G11,G12,G22
 *           (core/params.h:55-62, core/meshSetup.cpp:342-360)
 *   q, Aq   [fld*offset + e*Np + i + j*Nq + k*Nq*Nq]      (axhelm.okl:58-61)
 *   lambda  [id] = lambda0, [id+offset] = lambda1          (axhelm.okl:87-88)
 *   D       [i*Nq + m] = d l_m / dr at node i              (axhelm.okl:55)
 * Indices are 64-bit; gather ids are 32-bit like the reference's dlong.
 */
#ifndef NEKB_H
#define NEKB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
#define NEKB_OK                 0
#define NEKB_ERR_INVALID      (-1)  /* bad argument, size or handle                */
#define NEKB_ERR_CUDA         (-2)  /* a CUDA call failed                           */
#define NEKB_ERR_ALLOC        (-3)  /* device or host allocation failed             */
#define NEKB_ERR_UNSUPPORTED  (-4)  /* order / variant / precision not built        */
#define NEKB_ERR_BREAKDOWN    (-5)  /* Krylov breakdown (pAp <= 0 or non-finite)    */
#define NEKB_ERR_NOT_CONVERGED (-6) /* iteration limit reached before tolerance     */

/* axhelm variant bits: the name axhelm[Partial][_bk][_n3]_v0 of the reference
 * kernels (nekBone/setup.cpp:313-320, axhelm/main.cpp:105-109) maps to
 * PARTIAL | BK | N3. */
#define NEKB_AX_BK       1
#define NEKB_AX_N3       2
#define NEKB_AX_PARTIAL  4

/* precision of an axhelm application */
#define NEKB_FP64            0  /* ggeo/lambda/q/Aq double                                   */
#define NEKB_FP32            1  /* ggeo/lambda/q/Aq float                                    */
#define NEKB_BF16            2  /* ggeo and lambda bf16 storage, q/Aq float, FP32 arithmetic */
#define NEKB_FP32_TRILINEAR  3  /* geometry from 24 trilinear coefficients per element
                                   (float [E][24]) instead of ggeo; q/Aq/lambda float       */
#define NEKB_FP64_SPLIT      4  /* FP64 arrays as in NEKB_FP64, arithmetic on the FP32 pipes
                                   in double-float form (~48 bits; agrees with NEKB_FP64 to
                                   ~1e-14 relative); |values| < 3.4e38; no Partial forms    */

/* gather-scatter data types and ops (3rdParty/ogs/ogs.hpp:128-140) */
#define NEKB_DOUBLE 0
#define NEKB_FLOAT  1
#define NEKB_OP_ADD 0

const char* nekb_last_error(void);
int nekb_version(void);
int nekb_device_sync(void);
/* cudaMemcpy with the direction inferred from the pointers (helper for callers
 * that hold raw device pointers returned by this library) */
int nekb_copy(void* dst, const void* src, int64_t bytes);

/* ------------------------------------------------------------------ axhelm
 * Replaces the OCCA kernels axhelm_v0, axhelm_bk_v0, axhelm_n3_v0,
 * axhelm_bk_n3_v0 and their Partial forms (axhelm/kernel/VOLTA/axhelm.okl:28,
 * 158, 292, 484, 671, 865, 1063, 1188) as launched by
 *   kernel(Nelements, offset, o_ggeo, o_D, o_lambda, o_q, o_Aq)
 * (nekBone/solve.cpp:218, axhelm/main.cpp:132) and, with NEKB_AX_PARTIAL,
 *   kernel(Nelements, offset, o_elementList, o_ggeo, o_D, o_lambda, o_q, o_Aq)
 * (nekBone/solve.cpp:192-200).  Nq = N+1 in [2, 14] for NEKB_FP64 and [2, 12]
 * for the other precisions.  lambda may be NULL in BK
 * mode.  D is double for NEKB_FP64 and float otherwise.  All pointers are
 * device pointers. */
int nekb_axhelm(int Nq, int flags, int precision, int64_t Nelements, int64_t offset,
                const int32_t* elementList, const void* ggeo, const void* D, const void* lambda,
                const void* q, void* Aq, void* stream);

/* flags from a reference kernel name such as "axhelmPartial_bk_n3_v0"
 * (kernel naming of nekBone/setup.cpp:313-320, axhelm/main.cpp:105-109). */
int nekb_axhelm_flags_from_name(const char* name, int* flags);

/* Jacobi diagonal of the element Helmholtz operator before assembly; nodes
 * with mapB==1 get 1.  Replaces updateJacobi (nekBone/kernel/updateJacobi.okl:27).
 * mapB may be NULL (no masked nodes). */
int nekb_update_jacobi(int Nq, int64_t Nelements, int64_t offset, const int32_t* mapB,
                       const double* ggeo, const double* D, const double* lambda, double* diag,
                       void* stream);

/* ------------------------------------------------------------------ geometry
 * Second-order geometric factors from the element vertices (8 per element,
 * vertex order of core/meshSetup.cpp:2363-2410) for a trilinear map, at the
 * GLL nodes r1d with weights w1d; replaces meshGeometricFactorsHex3D
 * (core/meshSetup.cpp:215-360) for trilinear elements.  EX/EY/EZ, ggeo device
 * pointers (double); r1d, w1d host arrays of Nq. */
int nekb_geometric_factors(int Nq, int64_t Nelements, const double* EX, const double* EY,
                           const double* EZ, const double* r1d, const double* w1d, double* ggeo,
                           void* stream);
/* 24 trilinear coefficients per element ([e][c*8+a], float) used by the
 * NEKB_FP32_TRILINEAR operator. */
int nekb_trilinear_coeffs(int64_t Nelements, const double* EX, const double* EY, const double* EZ,
                          float* coef, void* stream);

/* 1D GLL / Gauss nodes and weights and the derivative matrix (host arrays);
 * restate meshJacobiGL, meshJacobiGQ and meshDmatrix1D (core/meshBasis.cpp:140,
 * 46, 775). */
int nekb_gll(int N, double* r, double* w);
int nekb_gauss(int N, double* r, double* w);
int nekb_dmatrix(int Nq, const double* r, double* D);

/* seeded uniform numbers in [lo,hi) (device), bit-identical to the CPU
 * generator used by the tests: value i = lo + (hi-lo)*u(seed, stream, i). */
int nekb_fill_uniform(double* v, int64_t n, uint64_t seed, uint64_t stream, double lo, double hi,
                      void* stream_);

/* ------------------------------------------------------------------ gather-scatter
 * Replaces ogsSetup(N, ids, comm, verbose, device) (3rdParty/ogs/ogs.hpp:178,
 * src/ogsSetup.cpp:68-355) on one rank: ids==0 nodes are excluded, groups are
 * numbered by first local appearance, members in ascending local index;
 * invDegree = 1/multiplicity.  ids is a HOST array of N global ids. */
typedef struct nekb_ogs nekb_ogs;
nekb_ogs* nekb_ogs_setup(int64_t N, const int64_t* ids, int verbose, int* status);
void nekb_ogs_free(nekb_ogs* ogs);
/* ogsGatherScatterMany(o_v, k, stride, type, op, ogs) (ogs.hpp:200) and
 * oogs::start/finish (ogs.hpp:259-260): sum over each group, written back to
 * every member, k fields at the given stride, fixed summation order. */
int nekb_ogs_gs_many(nekb_ogs* ogs, void* v, int k, int64_t stride, int dtype, int op,
                     void* stream);
/* sizes: [0]=N, [1]=Nlocal (ids!=0), [2]=NlocalGather, [3]=groups with >1 member */
int nekb_ogs_sizes(const nekb_ogs* ogs, int64_t* sizes4);
/* host copies of the CSR (offsets: NlocalGather+1, ids: Nlocal) for checking */
int nekb_ogs_copy_csr(const nekb_ogs* ogs, int32_t* offsets, int32_t* ids);
/* device pointer to invDegree (N doubles), owned by the handle (ogs->o_invDegree) */
const double* nekb_ogs_inv_degree(const nekb_ogs* ogs);

/* mask kernel (nekBone/kernel/utils.okl:127): q[maskIds[n]] = 0 */
int nekb_mask(int64_t Nmasked, const int32_t* maskIds, void* q, int dtype, void* stream);

/* ------------------------------------------------------------------ benchmark problem
 * Box mesh of nx*ny*nz hexahedra of order N on [box_min, box_max]^3 (the unit
 * cube when box_max <= box_min; the reference's default box is [-1,1]^3,
 * core/meshSetup.cpp:2316), interior vertices perturbed by
 * U[-perturb*h, perturb*h] (seeded), homogeneous Dirichlet on the boundary
 * (dirichlet=1) or periodic (periodic=1).  Builds on the device the
 * geometric factors, gather-scatter handle, mask list and solver workspace:
 * the state the reference keeps in mesh_t and BP_t (nekBone/BP.hpp:47-153,
 * nekBone/setup.cpp:36-367). */
typedef struct nekb_bp nekb_bp;
typedef struct {
  int N;
  int nx, ny, nz;
  int Nfields;        /* 1 or 3                                            */
  int periodic;       /* 1: periodic box (no boundary)                      */
  int dirichlet;      /* 1: boundary nodes masked (ids 0)                   */
  double perturb;     /* vertex perturbation fraction of h (0.1 typical)    */
  uint64_t seed;
  double box_min, box_max; /* extent per direction; box_max <= box_min: [0,1] */
} nekb_bp_config;

nekb_bp* nekb_bp_setup(const nekb_bp_config* cfg, void* stream, int* status);
/* The same state on the caller's own mesh, as the reference's setup() /
 * solveSetup() build it from mesh_t (nekBone/setup.cpp:36-367): ggeo (FP64,
 * reference layout, device or host, copied), global ids (host; 0 = not
 * assembled, ogs.hpp:42-44), the masked (Dirichlet) node list (host, may be
 * empty) and, optionally, the 8 vertices per element (host, vertex order of
 * core/meshSetup.cpp:2363-2410) for the trilinear-geometry inner operator
 * (NULL: NEKB_FP32_TRILINEAR is unavailable on this problem).  D is the GLL
 * derivative matrix of order N. */
nekb_bp* nekb_bp_setup_mesh(int N, int64_t Nelements, int Nfields, const double* ggeo,
                            const int64_t* ids, int64_t Nmasked, const int32_t* maskIds,
                            const double* EX, const double* EY, const double* EZ, void* stream,
                            int* status);
void nekb_bp_free(nekb_bp* bp);
/* sizes: [0]=Nq [1]=Nelements [2]=Np [3]=offset (Nlocal) [4]=Nmasked [5]=Nfields */
int nekb_bp_sizes(const nekb_bp* bp, int64_t* sizes6);
/* device pointers owned by the problem: name in {"ggeo","D","Df","invDegree",
 * "maskIds","EX","EY","EZ","x","y","z","trilinear"} */
void* nekb_bp_device_ptr(nekb_bp* bp, const char* name);
nekb_ogs* nekb_bp_ogs(nekb_bp* bp);

/* full operator used by the solvers: Aq = mask(gs(axhelm(q))) */
int nekb_bp_apply(nekb_bp* bp, int bk, int precision, const void* lambda, const void* q, void* Aq);

/* BPZeroMean(BP, o_q) (nekBone/solve.cpp:115-134): subtract from every entry
 * of q (device FP64, Nfields*offset) the mean of its Nelements*Np local values
 * over all fields (sum kernel utils.okl:212, addScalar utils.okl:29).
 * Deterministic fixed-order sum; runs on the problem's stream and returns
 * when it is done. */
int nekb_bp_zero_mean(nekb_bp* bp, double* q);

/* ------------------------------------------------------------------ PCG
 * BPPCG(BP, o_lambda, o_r, o_x, tol, MAXIT, opElapsed) (nekBone/solve.cpp:44-113,
 * nekBone/BP.hpp:172-178): r (in: rhs, out: residual) and x (in: guess, out:
 * solution) are device FP64 arrays of Nfields*offset; lambda device FP64
 * 2*offset (ignored when bk).  Stops when the invDegree-weighted |r|^2 <=
 * max(tol^2 |r0|^2, tol^2) (solve.cpp:85,90) or after maxit iterations. */
#define NEKB_PRECOND_COPY    0
#define NEKB_PRECOND_JACOBI  1
#define NEKB_PRECOND_LEARNED 2

#define NEKB_SOLVER_FP64     0   /* plain FP64 PCG (the reference algorithm)          */
#define NEKB_SOLVER_MIXED    1   /* FP32/BF16 inner PCG inside FP64 iterative refinement */
#define NEKB_SOLVER_FP64_SPLIT 2 /* the FP64 PCG with the double-float operator
                                    (NEKB_FP64_SPLIT; FP64 vectors and sums)       */

typedef struct {
  int solver;           /* NEKB_SOLVER_*                                        */
  int precond;          /* NEKB_PRECOND_*                                       */
  int flexible;         /* 1: flexible beta (KRYLOV SOLVER FLEXIBLE)            */
  int fixed_iterations; /* 1: run exactly maxit iterations                      */
  int bk;               /* 1: Poisson operator (lambda0=1, lambda1=0)           */
  int inner_precision;  /* NEKB_FP32 (default), NEKB_BF16 or NEKB_FP32_TRILINEAR
                           (mixed; the trilinear form keeps no FP32 geometry,
                           28 B/node less, at about 7 % more time)           */
  double inner_tol;     /* mixed: residual reduction between two replacements of
                           the FP32 residual by the true FP64 one (1e-2)       */
  int max_outer;        /* mixed: limit on FP64 residual replacements           */
  int check_every;      /* iterations between host convergence checks           */
  int use_graph;        /* 1: replay each chunk of iterations as a CUDA graph   */
  const void* net;      /* nekb_net* for NEKB_PRECOND_LEARNED                   */
  int zero_mean;        /* 1: nekb_bp_zero_mean on r before and on x after the
                           solve, as solve() does for an all-Neumann problem
                           (nekBone/main.cpp:24-31)                             */
  int fcg_window;       /* learned preconditioner: the new direction is made
                           A-orthogonal to the last fcg_window directions
                           (truncated flexible CG, FCG(m), 1..8; 0: 5).  A
                           nonlinear preconditioner needs m > 1: with m = 1
                           (the reference's flexible beta, solve.cpp:92-95)
                           conjugacy is lost over long solves              */
} nekb_pcg_opts;

typedef struct {
  int iterations;        /* BPPCG's return value (FP32 Krylov iterations, mixed) */
  int outer_iterations;  /* FP64 true-residual evaluations (mixed; 1 for FP64)   */
  int status;            /* NEKB_OK, NEKB_ERR_BREAKDOWN, NEKB_ERR_NOT_CONVERGED  */
  double rdotr0;         /* weighted |r0|^2                                      */
  double rdotr;          /* weighted |r|^2 of the last check                     */
  double true_rel_res;   /* |b - A x|_w / |b|_w in FP64 after the solve          */
  double elapsed_s;      /* device time of the solve                             */
} nekb_pcg_stats;

/* BPWeightedInnerProduct(BP, o_w, o_a, o_b) (nekBone/solve.cpp:237-259) with the
 * weightedMultipleInnerProduct2 kernel (nekBone/kernel/utils.okl:413-458):
 * *wab = sum over the Nfields fields of w[i] a[i+f*offset] b[i+f*offset]
 * (w device, Nlocal entries; a, b device, Nfields*offset).  Deterministic
 * fixed-order reduction on the problem's own scratch; result on the host. */
int nekb_bp_weighted_inner_product(nekb_bp* bp, const double* w, const double* a, const double* b,
                                   double* wab);
/* BPWeightedInnerProduct2 (nekBone/solve.cpp:261-287) with weightedInnerProductUpdate
 * (nekBone/kernel/utils.okl:687-793): wab2[0] = sum w a b, wab2[1] = sum w a a. */
int nekb_bp_weighted_inner_product2(nekb_bp* bp, const double* w, const double* a,
                                    const double* b, double* wab2);

/* The same weighted inner product for callers that cannot allocate device
 * memory: an application whose GPU memory all belongs to its own pool
 * allocator, or a loop that must not trigger the implicit synchronisation a
 * cudaMalloc can cause.  No counterpart in the reference.
 * *wab (a device double) = sum over the Nfields fields of w[i] a[i+f*offset]
 * b[i+f*offset], i < N, computed on the given stream; nothing is allocated.
 * The scratch (one partial sum per 256-node block and a completion ticket) is
 * a fixed 1 MiB array inside the library, held by every GPU that loads the
 * library until the process exits; N above 33,554,432 nodes per field is
 * refused with NEKB_ERR_INVALID.  Every call shares that array, so calls that
 * overlap on the same GPU race.  The first call on a device looks up the
 * array's device address and keeps it for the life of the process; make it
 * before any stream capture.  A device reset (cudaDeviceReset) is not
 * supported for this entry point: the kept address would be stale. */
int nekb_weighted_inner_product_noalloc(int64_t N, int Nfields, int64_t offset, const double* w,
                                        const double* a, const double* b, double* wab,
                                        void* stream);

/* ------------------------------------------------------------------ dot benchmark */
/* The dot benchmark's kernels (dot/kernel/VOLTA/dot.okl), launched by the
 * driver as kernel(N, o_w, o_x, o_y, o_tmp) (dot/main.cpp:27-48, 123-126):
 * wxy[b] (device, nekb_dot_num_blocks(N, blockSize) doubles) = the sum over
 * block b of blockSize consecutive nodes, reduced in the reference kernel's
 * own tree, so every partial is bit-for-bit the reference's; the caller sums
 * the partials (the driver does it on the host in block order).
 *   variant 0: weightedInnerProduct2_v0 (dot.okl:27-65), w[i] x[i] y[i],
 *              blockSize = p_blockSize (256, 512 or 1024);
 *   variant 1: weightedInnerProduct2_v1 (dot.okl:114-169), blocks of 256
 *              nodes reduced as 8 groups of 32 (the lockstep tree);
 *   variant 2: weightedBlockInnerProduct2 (dot.okl:67-111), per node the sum
 *              over Nfields (p_eNfields, 1..3) of w x y at i + f*offset.
 * N = 0 writes nothing.  Asynchronous on the stream. */
int64_t nekb_dot_num_blocks(int64_t N, int blockSize);
int nekb_dot_partials(int variant, int64_t N, int Nfields, int64_t offset, int blockSize,
                      const double* w, const double* x, const double* y, double* wxy,
                      void* stream);

/* ------------------------------------------------------------------ adv benchmark */
/* advCubatureHex3D_v0 (adv/kernel/VOLTA/adv.okl:27-261), launched as
 * kernel(Nelements, o_vgeo, o_cubvgeo, o_cubD, o_cubInterpT, offset, o_U, o_NU)
 * (adv/main.cpp:115-123), FP64: the dealiased advection term of the velocity
 * U (3 fields, field f at U + f*offset, node i + Nq j + Nq^2 k of element e at
 * e*Nq^3 + ...):
 *   NU_f = IJW . (I^T x I^T x I^T) [Uhat dUc_f/dr + Vhat dUc_f/ds + What dUc_f/dt],
 *   Uc = (I x I x I) U,  Uhat = JW (Uc . grad r), Vhat = JW (Uc . grad s), What = JW (Uc . grad t)
 * with I(i <- a) = cubInterpT[a*cubNq + i] (Nq x cubNq), the cubature
 * derivative cubD[i*cubNq + n] (cubNq x cubNq), the metric slots RX..TZ and JW
 * of cubvgeo (12 slots of cubNq^3 per element) and IJW of vgeo (12 slots of
 * Nq^3), slot numbers of core/params.h:2-13.  Built for cubNq = Nq (Nq 2..12)
 * and cubNq = ceil(3 Nq / 2) (Nq 2..10); NEKB_ERR_UNSUPPORTED otherwise.
 * precision: NEKB_FP64 (native FP64 FMAs; the reference's dfloat = double) or
 * NEKB_FP64_SPLIT (the same FP64 arrays, arithmetic in double-float on the
 * FP32 pipes: within ~1e-13 relative of FP64, values in the float range).
 * For cubNq > Nq the reference kernel indexes its Nq x Nq shared tile s_U with
 * cubNq x cubNq indices (adv.okl:203-231); this operator uses a cubNq x cubNq
 * slice there (the two agree for cubNq = Nq).  Asynchronous on the stream. */
int nekb_adv_cubature(int Nq, int cubNq, int precision, int64_t Nelements, const double* vgeo,
                      const double* cubvgeo, const double* cubD, const double* cubInterpT,
                      int64_t offset, const double* U, double* NU, void* stream);

void nekb_pcg_default_opts(nekb_pcg_opts* opts);
int nekb_bp_pcg(nekb_bp* bp, const double* lambda, double* r, double* x, double tol, int maxit,
                const nekb_pcg_opts* opts, nekb_pcg_stats* stats);

/* ------------------------------------------------------------------ learned preconditioner
 * Per-element 3D convolution network: layers of 3x3x3 convolutions on the Nq^3
 * nodes of each element (zero padding at the element boundary), channels
 * 1 -> C -> ... -> C -> 1, tanh-form GELU between layers, BF16 weights with
 * FP32 accumulation.  Used inside flexible PCG as
 *   z = invDiag*r + mask(gs(invDegree * h * s_e * net(h * r_e / s_e)))
 * with h = sqrt(invDiag) per node and s_e the RMS of h*r over element e.
 * No counterpart in the reference. */
typedef struct nekb_net nekb_net;
nekb_net* nekb_net_create(int Nq, int channels, int layers, uint64_t seed, int* status);
/* inference arithmetic: NEKB_NET_TENSOR (default: BF16 tensor-core MMAs with
 * BF16 activations between layers and FP32 sums, on the library's preferred
 * tensor-core kernel; built for Nq=8 with 16 channels, other shapes fall back
 * to NEKB_NET_FP32), NEKB_NET_TENSOR_SYNC (that arithmetic on warp-level
 * mma.sync instructions), NEKB_NET_TENSOR_TC5 (that arithmetic on tcgen05
 * MMAs with accumulators in tensor memory) or NEKB_NET_FP32 (FP32 activations
 * and sums on the CUDA cores).  nekb_net_inference returns the mode in use
 * (NEKB_NET_FP32 where a tensor-core mode is not built for the shape). */
#define NEKB_NET_FP32        0
#define NEKB_NET_TENSOR      1
#define NEKB_NET_TENSOR_SYNC 2
#define NEKB_NET_TENSOR_TC5  3
int nekb_net_set_inference(nekb_net* net, int mode);
int nekb_net_inference(const nekb_net* net);
void nekb_net_free(nekb_net* net);
int nekb_net_num_params(const nekb_net* net);
/* FP32 master weights (host arrays of nekb_net_num_params floats) */
int nekb_net_get_weights(const nekb_net* net, float* w);
int nekb_net_set_weights(nekb_net* net, const float* w);
/* forward on E element blocks: in/out device float [E][Nq^3]; with the
 * tensor-core inference the arrays must be 16-byte aligned (whole element rows
 * are fetched by bulk copies) and the call returns once the stream is done */
int nekb_net_forward(nekb_net* net, int64_t E, const float* in, float* out, void* stream);
/* Sets, from the host, the flag the tensor-core network kernel raises when its
 * bulk input copies do not arrive within its bounded wait.  The next
 * nekb_net_forward or learned solve then returns NEKB_ERR_CUDA ("did not
 * complete in time") and clears the flag.  For tests of that error path: no
 * device wait has to run out.  No counterpart in the reference. */
int nekb_net_raise_copy_timeout(void);
/* one training step on a batch: loss = mean_e |net(in_e) - target_e|^2 / Np;
 * computes gradients with the network's own backward kernels and applies Adam.
 * loss (host) may be NULL. */
int nekb_net_train_step(nekb_net* net, int64_t E, const float* in, const float* target, float lr,
                        float* loss, void* stream);
/* gradient of the loss w.r.t. the FP32 master weights (host float array), no update */
int nekb_net_gradient(nekb_net* net, int64_t E, const float* in, const float* target, float* grad,
                      float* loss, void* stream);
/* training pairs from solver snapshots: per element e, h = sqrt(invDiag) per
 * node, s_e = RMS of h*r_e, in_e = h*r_e / s_e and target_e =
 * (err_e - invDiag*r_e) / (h s_e) (device float arrays of E*Np; invDiag of
 * Efield*Np may be NULL, then h = 1 and the Jacobi term is dropped) */
int nekb_net_prepare_pairs(int Np, int64_t E, int64_t Efield, const float* r, const float* err,
                           const float* invDiag, float* in, float* target, void* stream);
/* Element-local correction y of n residual rows r (device FP32, [n][Np], row b
 * taken from element elems[b] of field 0): on the element-interior nodes the
 * solution of the element's Helmholtz problem A_II y_I = r_I with y = 0 on the
 * element boundary (FP32 CG, at most iters steps, relative tolerance tol); on
 * the element-boundary nodes invDiag*r (invDiag rows [n][Np]).  lambda as in
 * nekb_bp_pcg (2*offset FP64).  Training target for the learned
 * preconditioner (with nekb_net_prepare_pairs, err = y); an element index
 * outside the mesh gives a zero row.  Runs on the problem's stream and returns
 * when it is done.  Nq 3..8.
 * No counterpart in the reference. */
int nekb_bp_local_correction(nekb_bp* bp, const double* lambda, const int32_t* elems, int64_t n,
                             const float* r, const float* invDiag, float* y, int iters, float tol);
/* versioned checkpoint (header, sizes, step, weights, Adam moments, CRC-32) */
int nekb_net_save(const nekb_net* net, const char* path);
nekb_net* nekb_net_load(const char* path, int* status);

/* ------------------------------------------------------------------ microbenchmarks */
/* FP64 / FP32 FMA throughput and HBM copy bandwidth of the current device */
int nekb_peak_fma(int fp64, double* tflops);
int nekb_peak_copy(double* gbs);

#ifdef __cplusplus
}
#endif
#endif
