/* dcpse_capi.h -- C-ABI of the GB300 DC-PSE hot path.
 *
 * Plain C: POD arguments, device pointers (d_*) or host pointers (h_*), an
 * opaque plan handle, int status.  No C++ or torch types cross this line.
 * The C++ drop-in headers (Dcpse.hpp, DCPSE_op.hpp in this directory) and the
 * Python package call these symbols.
 *
 * Citations are to the openfpm_numerics source tree (src/...).
 *
 * Threading: a plan is not thread-safe; every call is enqueued on the plan's
 * stream (default: the legacy default stream) and calls that return data to
 * the host synchronise that stream.
 *
 * Array sizes: fields, outputs and positions are bare pointers whose lengths
 * follow from the plan (n domain particles from the neighbour list, n_support
 * for support-set fields, n_outputs), as the reference's own property
 * vectors do; a shorter array is read or written out of bounds.  The C++ and
 * Python mirrors check the lengths before calling.
 */
#ifndef OPENFPM_DCPSE_CAPI_H
#define OPENFPM_DCPSE_CAPI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define DCPSE_OK 0
#define DCPSE_ERR_ARG 1        /* invalid argument */
#define DCPSE_ERR_CUDA 2       /* CUDA runtime error (dcpse_last_error has it) */
#define DCPSE_ERR_STATE 3      /* call out of order (e.g. apply before assemble) */
#define DCPSE_ERR_CAPACITY 4   /* a size limit was exceeded */
#define DCPSE_ERR_IO 5         /* save/load failure */
#define DCPSE_ERR_PARTICLES 6  /* some particles could not be assembled */
#define DCPSE_ERR_TIMEOUT 7    /* a bounded device wait ran out (results invalid) */

/* per-particle assembly status (dcpse_particle_status / status arrays).
 * The reference raises std::length_error for too few neighbours
 * (src/DCPSE/Vandermonde.hpp:109-112) and asserts eps != 0
 * (src/DCPSE/Vandermonde.hpp:80); here the particle's weights are zero and
 * the code below is recorded. */
#define DCPSE_PART_OK 0
#define DCPSE_PART_TOO_FEW 1   /* fewer neighbours than basis functions */
#define DCPSE_PART_BAD_EPS 2   /* eps not finite or not > 0 */
#define DCPSE_PART_SINGULAR 3  /* zero pivot column in the moment matrix */
#define DCPSE_PART_NONFINITE 4 /* non-finite kernel value */

/* store flags of dcpse_assemble */
#define DCPSE_STORE_TERMS_F64 1 /* per reference Dcpse object: calcKernels + localEpsInvPow, FP64 */
#define DCPSE_STORE_OUT_F64 2   /* per output, terms summed, eps^-|alpha| folded in, FP64 */
#define DCPSE_STORE_OUT_F32 4   /* per output, terms summed, eps^-|alpha| folded in, FP32 */
#define DCPSE_ASSEMBLE_FAST 8   /* outputs from summed right-hand sides (one solve
                                   per output and basis) instead of per-term sums */
#define DCPSE_ASSEMBLE_ASYNC 16 /* do not synchronise; query dcpse_particle_status */
#define DCPSE_STORE_OUT_F32_RESID 32 /* also bf16 residuals w64 - w32 of the FP32 weights */
#define DCPSE_STORE_OUT_F32_CORR 64  /* also FP32 residuals w64 - w32 (for DCPSE_F32_BUDGET) */
#define DCPSE_ASSEMBLE_TC 128   /* with DCPSE_ASSEMBLE_FAST: the Gram products B^T B on the tensor
                                   cores (tcgen05), from a 62-bit fixed-point B: not bit-identical
                                   to the sequential FP64 sums, closer to the correctly rounded
                                   Gram than they are; taken when the union basis has <= 24
                                   functions and no row has more than 128 neighbours, else the
                                   FP64 kernel serves (dcpse_plan_assembly_info tells which) */

/* precision of dcpse_apply_batched */
#define DCPSE_F64 0
#define DCPSE_F32 1       /* FP32 weights, exact differences, compensated sums */
#define DCPSE_F32_RESID 2 /* FP32 weights + bf16 residual correction (near-FP64 accuracy) */
#define DCPSE_F32_BUDGET 3 /* FP32 weights, then an FP64 residual correction of exactly the
                              rows whose FP32 error bound exceeds the plan's error budget */
#define DCPSE_F32_PAIR 4   /* weights as FP32 pairs w32 + (w64 - w32) (48 bits), the field in 62-bit
                              fixed point (one power-of-two scale from the call's largest |f|: exact
                              differences f_q - f_p), compensated FP32 sums: FP64-class results
                              (<= 1e-12 normwise) at the FP64 weights' bytes, off the FP64 pipe.
                              A NaN or an infinity in the field makes every output NaN.  Needs
                              DCPSE_STORE_OUT_F32 | DCPSE_STORE_OUT_F32_CORR; without the sliced
                              layout the batched FP64 apply serves.  Batched applies only. */

typedef struct dcpse_plan_s dcpse_plan_t;

/* Last error message of this thread ("" if none). */
const char* dcpse_last_error(void);
int dcpse_version(void);

/* ---- plan ---------------------------------------------------------------
 * A plan holds one particle set (domain == support), its neighbour list and
 * n_outputs operators.  Output o is the sum of terms_per_output[o] reference
 * Dcpse objects whose signatures follow in `signatures` (dim entries each):
 *   Derivative_x   1 term  (1,0[,0])     src/DCPSE/DCPSE_op/DCPSE_op.hpp:666-679
 *   Derivative_xx  1 term  (2,0[,0])     DCPSE_op.hpp:2216-2358
 *   Laplacian      dim terms 2e_i        DCPSE_op.hpp:1367-1389 (VECT_DCPSE_V_SUM :388-399)
 *   Gradient       dim outputs of e_i    DCPSE_op.hpp:1099-1120 (VECT_DCPSE_V :144-153)
 * order = convergence order, h_over_eps = Dcpse::HOverEpsilon (Dcpse.hpp:80,
 * 0.9 in the reference CPU path; the reference GPU path's eps = 2 <h>
 * (Dcpse.cuh:799-807) corresponds to 0.5).
 * Replaces: Dcpse::Dcpse (src/DCPSE/Dcpse.hpp:91-109) and the operator
 * constructors above, minus the assembly itself. */
int dcpse_plan_create(dcpse_plan_t** plan, int dim, int n_outputs, const int* terms_per_output,
                      const unsigned* signatures, unsigned order, double h_over_eps);
int dcpse_plan_destroy(dcpse_plan_t* plan);
/* stream: a cudaStream_t (NULL = legacy default stream) */
int dcpse_plan_set_stream(dcpse_plan_t* plan, void* stream);
/* Domain box and periodicity (minimum-image offsets along periodic axes).
 * Without a box the neighbour search uses the particles' bounding box and no
 * axis is periodic.  Replaces the ghost layer the reference gets from
 * vector_dist::ghost_get (Dcpse.hpp:107). */
int dcpse_plan_set_box(dcpse_plan_t* plan, const double* lo, const double* hi, const int* periodic);
/* Support set of the neighbour lists (the columns).  With d_pos_support
 * non-NULL the plan is a two-set operator: rows are the domain particles
 * passed to dcpse_build_neighbors / dcpse_assemble, columns index the n_support
 * support particles, and no entry is skipped (Dcpse's two-set constructor,
 * Dcpse.hpp:113-131, as used by PPInterpolation, DcpseInterpolation.hpp:
 * 55-81, with createVerletTwoPhase lists).  With NULL the domain set is its
 * own support and self_skip selects VL_SKIP_REF_PART (1, the default) or a
 * plain VL_NON_SYMMETRIC list that holds the particle itself (0).  The plan
 * keeps the pointer, as the reference keeps a reference to the set; the
 * neighbour list is dropped (build it again).  Derivative applies, adjoints
 * and RK4 stages need one set and return DCPSE_ERR_STATE on two. */
int dcpse_plan_set_support(dcpse_plan_t* plan, const double* d_pos_support, int64_t n_support, int self_skip);
/* Surface DC-PSE (SurfaceDcpse, Dcpse.hpp:829-1085; the surface operators of
 * DCPSE_surface_op.hpp and PPInterpolation's surface form).  With d_normals
 * non-NULL (unit normals [n_base][dim] of the support set: the domain set, or
 * the second set of dcpse_plan_set_support), dcpse_build_neighbors extends
 * the support by 2*n_count virtual particles per base particle p at
 * x_p +- (i s_p) n_p, i = 1..n_count (createNormalParticles, Dcpse.hpp:855-
 * 876), s_p = d_n_spacings[p] if given (support_options::ADAPTIVE) else
 * n_spacing; dcpse_assemble then assembles on the extended support and adds
 * every virtual particle's kernels onto its base particle
 * (accumulateAndDeleteNormalParticles, Dcpse.hpp:947-1015): the neighbour
 * list holds each base particle once, in order of first appearance.  The
 * plan keeps the pointers; each assembly needs its own neighbour build.
 * NULL normals switch surface mode off.  The neighbour list is dropped. */
int dcpse_plan_set_surface(dcpse_plan_t* plan, const double* d_normals, int n_count, double n_spacing,
                           const double* d_n_spacings);
/* sizes: n particles, nnz neighbour entries, terms, outputs, max neighbours */
int dcpse_plan_info(dcpse_plan_t* plan, int64_t* n, int64_t* nnz, int* n_terms, int* n_outputs,
                    int* max_neighbors);
/* Basis of term t (MonomialBasis, src/DCPSE/MonomialBasis.hpp:114-157):
 * exps gets n x dim exponents (n <= cap), returns n through *n. */
int dcpse_term_basis(dcpse_plan_t* plan, int term, unsigned* exps, int cap, int* n);

/* ---- neighbour lists ----------------------------------------------------
 * CSR lists, ascending neighbour index, self excluded, |x_p - x_q|^2 < rc^2
 * with rc = d_rcut_pp[p] when given (per-particle radius, the adaptive
 * support of Dcpse.hpp:903-909) else rcut.
 * Replaces: VerletList getVerlet<VL_NON_SYMMETRIC|VL_SKIP_REF_PART>(rCut)
 * (e.g. src/DCPSE/tests/Dcpse_unit_tests.cpp:97) and SupportBuilderGPU
 * (src/DCPSE/SupportBuilder.cuh:14-107, device-only here: no host scan). */
int dcpse_build_neighbors(dcpse_plan_t* plan, const double* d_pos, int64_t n, double rcut,
                          const double* d_rcut_pp);
/* Use a caller-built list (e.g. the caller's own VerletList exported to CSR).
 * The arrays are copied. */
int dcpse_set_neighbors(dcpse_plan_t* plan, int64_t n, int64_t nnz, const int64_t* d_rowptr,
                        const int32_t* d_cols);
int dcpse_neighbors_ptr(dcpse_plan_t* plan, const int64_t** d_rowptr, const int32_t** d_cols);

/* ---- assembly -----------------------------------------------------------
 * Builds eps, eps^-|alpha| and the kernels of every term (and/or the summed
 * output weights) for all particles on the device, in FP64.
 * d_eps_fixed: optional per-particle eps override (NULL = reference eps).
 * Returns DCPSE_ERR_PARTICLES if any particle failed (see
 * dcpse_particle_status); the plan is still usable, failed rows are zero.
 * Replaces: Dcpse::initializeStaticSize (src/DCPSE/Dcpse.hpp:690-796),
 * Dcpse_gpu::assembleLocalMatrices (src/DCPSE/Dcpse.cuh:620-717). */
int dcpse_assemble(dcpse_plan_t* plan, const double* d_pos, const double* d_eps_fixed, int flags);
/* Whether the last assembly took its Gram products on the tensor cores
 * (DCPSE_ASSEMBLE_TC). */
int dcpse_plan_assembly_info(dcpse_plan_t* plan, int* gram_on_tensor_cores);
int dcpse_particle_status(dcpse_plan_t* plan, int64_t* n_bad, int64_t* first_bad, int* first_code);
/* Device arrays owned by the plan (valid until the next assemble/destroy). */
int dcpse_eps_ptr(dcpse_plan_t* plan, const double** d_eps, const int32_t** d_status);
/* calcKernels / localEpsInvPow of term t (Dcpse.hpp:59-63), FP64 */
int dcpse_term_kernels_ptr(dcpse_plan_t* plan, int term, const double** d_kernels,
                           const double** d_eps_inv_pow);
/* summed, eps-folded output weights (either may be NULL if not stored) */
int dcpse_output_weights_ptr(dcpse_plan_t* plan, int output, const double** d_w64, const float** d_w32);
/* Installs previously saved kernels of term t (calcKernels[nnz], localEps[n],
 * localEpsInvPow[n], device pointers, copied) on a plan whose neighbour list
 * is set; the plan then counts as assembled for the per-term FP64 entry
 * points (summed output weights of an earlier assembly are dropped).
 * Replaces: Dcpse::load (src/DCPSE/Dcpse.hpp:337-379). */
int dcpse_set_term_kernels(dcpse_plan_t* plan, int term, const double* d_kernels, const double* d_eps,
                           const double* d_eps_inv_pow);

/* ---- device memory helpers ----------------------------------------------
 * So that host code above this ABI needs no CUDA headers.  Replace the role
 * of openfpm_devices' CudaMemory (hostToDevice / deviceToHost). */
int dcpse_device_alloc(void** ptr, uint64_t bytes);
int dcpse_device_free(void* ptr);
/* Page-locked host memory mapped into the device address space: host
 * buffers that dcpse_apply_batched_host reads and writes in place. */
int dcpse_host_alloc(void** ptr, uint64_t bytes);
int dcpse_host_free(void* ptr);
/* synchronous copy between any host / device pointers */
int dcpse_copy(void* dst, const void* src, uint64_t bytes);

/* ---- apply --------------------------------------------------------------
 * Df_p = eps_p^-|alpha| sum_q (f_q + s f_p) K_pq, s = -1 for even |alpha|,
 * in the reference's operation order (bit-exact with it).
 * Replaces: Dcpse::computeDifferentialOperator<f,Df> (src/DCPSE/Dcpse.hpp:467-499)
 * and the per-key form (Dcpse.hpp:560-603). */
int dcpse_apply_term_f64(dcpse_plan_t* plan, int term, const double* d_f, double* d_out);
/* Output o as the reference composes it (sum of its terms, VECT_DCPSE_V_SUM,
 * DCPSE_op.hpp:388-399), FP64, one term after the other. */
int dcpse_apply_output_f64(dcpse_plan_t* plan, int output, const double* d_f, double* d_out);
/* All outputs in one pass over the neighbour list from the summed weights:
 * d_out[o*n + p] = sum_q w_o,pq (f_q - f_p).  precision DCPSE_F32 uses the
 * FP32 weights with FP32 arithmetic, DCPSE_F64 the FP64 ones.
 * Replaces the host loop vector_dist_op_compute_op<prp,comp_host>::compute_expr
 * (src/Operators/Vector/cuda/vector_dist_operators_cuda.cuh:444-461) for
 * `getV<j>(parts) = Op(getV<i>(parts))`. */
int dcpse_apply_batched(dcpse_plan_t* plan, const double* d_f, double* d_out, int precision);
/* Same with host buffers h_f[n], h_out[n_outputs*n]: the copies are part of
 * the call (the reference's bulk apply reads and writes host particles). */
int dcpse_apply_batched_host(dcpse_plan_t* plan, const double* h_f, double* h_out, int precision);

/* Error budget of DCPSE_F32_BUDGET applies (default 1e-6): every output o
 * of the call satisfies
 *     max_p |out_o,p - out64_o,p| <= budget * max_p |out64_o,p|
 * against the FP64 summed weights out64 (DCPSE_F64).  The FP32 kernel bounds
 * each row's weight-rounding error, 2^-24 sum_q |w32_o,pq| |f_q - f_p|, and
 * a second pass adds sum_q (w64 - w32)_o,pq (f_q - f_p) in FP64 to exactly
 * the rows whose bound exceeds budget/2 of the call's largest |output|.
 * Needs DCPSE_STORE_OUT_F32_CORR at assembly.  first_pass DCPSE_F32 (the
 * default) streams the FP32 weights alone: the cheapest when few rows need
 * the second pass (smooth fields on near-uniform sets).  DCPSE_F32_RESID
 * also streams the bf16 residuals (DCPSE_STORE_OUT_F32_RESID at assembly):
 * its bound shrinks to 2^-32 sum_q ..., so far fewer rows need the second
 * pass (second derivatives on strongly graded clouds).  Floor: a corrected row is exact to about 2^-48 sum_q
 * |w| |f_q - f_p|, the order of the FP64 apply's own rounding, so budgets
 * below that relative to max|out| (e.g. outputs that vanish identically)
 * cannot be resolved.  The reference stores its
 * weights in FP64 only (Dcpse.hpp:59-63, applied at Dcpse.hpp:467-499); this
 * is how the FP32 weights keep to its results.  budget in (0, 1). */
int dcpse_plan_set_error_budget(dcpse_plan_t* plan, double budget, int first_pass);
/* (row, output) pairs the DCPSE_F32_BUDGET applies corrected since the last
 * reset (synchronises the plan's stream; reset != 0 zeroes the count). */
int dcpse_plan_budget_stats(dcpse_plan_t* plan, int64_t* pairs_corrected, int reset);

/* Particle numbering of the batched applies' sliced layout.  The apply
 * gathers f_q for every neighbour q; in the caller's numbering those reads
 * are local only if the caller's particles are stored in spatial order.  A
 * neighbour list built by dcpse_build_neighbors (one particle set) carries
 * the particles' cell order, and the layout built at assembly renumbers rows
 * and columns by it when the caller's numbering scatters the reads at least
 * twice as far (mean |q - p| over the entries against the cell order's),
 * policy 0 (default); policy 1 always renumbers, -1 never.  Results are the
 * same bit for bit either way (each row keeps its entries' order); outputs
 * stay in the caller's numbering.  The reference's GPU support builder walks
 * particles cell by cell for the same reason (SupportBuilder.cuh:14-61).
 * Applies on row ranges, RK4 stages and p2p keep the caller's numbering
 * (CSR kernels) on a renumbered layout.  Changing the policy rebuilds the
 * layout. */
int dcpse_plan_set_reorder(dcpse_plan_t* plan, int policy);
/* The renumbering order the next dcpse_build_neighbors computes: 0 (default)
 * the Z-order of the list's cells, 1 row-major order of a grid at the
 * particles' mean spacing.  No counterpart in the reference. */
int dcpse_plan_set_reorder_order(dcpse_plan_t* plan, int order);
/* Whether the current layout is renumbered, and the mean |q - p| of the
 * list's entries in the caller's numbering and in the cell order (0 when no
 * cell order is known: caller-built lists, two sets, surface operators). */
int dcpse_plan_reorder_info(dcpse_plan_t* plan, int* renumbered, double* mean_dist_list, double* mean_dist_cells);

/* ---- particle to particle interpolation --------------------------------
 * Replaces Dcpse::p2p<prp1,prp2>() and p2p<prp1,prp2,N1>() (Dcpse.hpp:198-
 * 297) behind PPInterpolation::p2p (DcpseInterpolation.hpp:133-160): for every
 * domain particle p and component c,
 *     out[p*ncomp + c] = epsInvPow_p * sum_q f[q*ncomp + c] K_pq
 * with f on the support set (no f_p term).  dcpse_p2p_f64 uses the per-term
 * FP64 kernels in the reference's order (DCPSE_STORE_TERMS_F64);
 * dcpse_p2p applies every output at once from the summed weights, FP64 or
 * FP32 (field as an exact float pair), out[o*n*ncomp + p*ncomp + c]. */
int dcpse_p2p_f64(dcpse_plan_t* plan, int term, const double* d_f_support, int ncomp, double* d_out);
int dcpse_p2p(dcpse_plan_t* plan, const double* d_f_support, int ncomp, double* d_out, int precision);

/* ---- operator matrices --------------------------------------------------
 * CSR rows of output `output` times coeff, as DCPSE_scheme::impose builds
 * them from value_nz (DCPSE_op.hpp:70-83, :405-420; DCPSE_Solver.hpp:980-
 * 1030): for row r (particle p = d_rows[r], or r when d_rows is NULL and
 * n_rows is ignored), column q*nvar + var holds sum_terms (K_pq * coeff) *
 * epsInvPow_p and column p*nvar + var the diagonal sum_terms sum_q
 * ((sign * K_pq) * coeff) * epsInvPow_p with Dcpse::getSign(), accumulated in
 * the reference's order; columns ascending, a zero diagonal for a row
 * without neighbours.  Two calls: with d_cols_out = d_vals_out = NULL it
 * writes d_rowptr_out[n_rows+1] (device) and *nnz_out (host); then with
 * arrays of *nnz_out entries it fills them.  Needs DCPSE_STORE_TERMS_F64. */
int dcpse_operator_csr(dcpse_plan_t* plan, int output, double coeff, const int64_t* d_rows, int64_t n_rows, int nvar,
                       int var, int64_t* d_rowptr_out, int64_t* d_cols_out, double* d_vals_out, int64_t* nnz_out);

/* ---- adjoint ------------------------------------------------------------
 * No counterpart in the reference (its operators have no derivatives); these
 * differentiate the batched apply y_o = L_o f with the neighbour list held
 * fixed.
 * Field VJP: d_out[q] = sum_o (L_o^T g_o)_q for a cotangent d_g[o*n + p],
 * from the FP64 (DCPSE_F64) or FP32 (DCPSE_F32) output weights, through a
 * transposed neighbour list built once per list (fixed summation order). */
int dcpse_vjp_field(dcpse_plan_t* plan, const double* d_g, double* d_out, int precision);
/* Position VJP: d_grad[i*dim + d] = d/dx_i,d of sum_o,p g_o,p (L_o f)_p,
 * differentiating through every particle's moment-matrix solve, eps and the
 * scaling eps^-|alpha| (FP64).  d_pos must be the positions the plan was
 * assembled with; d_eps_fixed the override used there, or NULL. */
int dcpse_vjp_positions(dcpse_plan_t* plan, const double* d_pos, const double* d_eps_fixed, const double* d_f,
                        const double* d_g, double* d_grad);

/* ---- RK4 time stepping of two-species reaction-diffusion ----------------
 * Gray-Scott:  du = Du L u - u v^2 + F (1 - u),  dv = Dv L v + u v^2 - (F+k) v
 * with L = output 0 of the plan (a Laplacian; FP32 weights for
 * precision DCPSE_F32 with float state arrays, FP64 output weights for
 * DCPSE_F64 with double arrays).  params = {Du, Dv, F, k, dt}.
 * One call is one classic RK4 stage (stage 0..3; see dcpse_rk4.cu for the
 * buffers each stage reads and writes); four calls make a step and contain
 * no synchronisation or allocation, so a step can be captured in a CUDA
 * graph.  Replaces: boost odeint runge_kutta4 over the DC-PSE Laplacian as
 * used in src/OdeIntegrators/tests/OdeIntegratores_base_tests.cpp:33-72,478-577. */
int dcpse_rk4_gs_stage(dcpse_plan_t* plan, int stage, int precision, const void* Yu, const void* Yv, const void* y0u,
                       const void* y0v, void* accu, void* accv, void* outu, void* outv, const double* params);
/* Builds the transposed Laplacian weights used by the adjoint stages
 * (call after assembly, outside graph capture). */
int dcpse_rk4_gs_adjoint_prepare(dcpse_plan_t* plan, int precision);
/* One reverse RK4 stage: acc += J(Y)^T kbar; next = cy * ybar + cY * J(Y)^T kbar
 * (next may be NULL).  params = {Du, Dv, F, k, dt}. */
int dcpse_rk4_gs_adjoint_stage(dcpse_plan_t* plan, int precision, const void* Yu, const void* Yv, const void* kbu,
                               const void* kbv, const void* ybu, const void* ybv, void* accu, void* accv, void* next_u,
                               void* next_v, double cy, double cY, const double* params);
/* One whole reverse RK4 step: ybar (ybu, ybv) of y_(n+1) is replaced by ybar
 * of y_n, from the step's stage states stages = {Y1u, Y1v, Y2u, Y2v, Y3u,
 * Y3v, Y4u, Y4v}; acc (accu, accv) is work space.  The same arithmetic as
 * the four adjoint stages with their kbar scalings and copies, bit for bit,
 * in five kernels (kbar kept as pairs, the accumulator started and handed
 * back by the first and last stage).  No synchronisation or allocation. */
int dcpse_rk4_gs_reverse_step(dcpse_plan_t* plan, int precision, const void* const* stages, void* ybu, void* ybv,
                              void* accu, void* accv, const double* params);

/* ---- batched FP32 apply that allocates nothing --------------------------
 * No counterpart in the reference.  For callers that must not allocate
 * device memory: code running inside an allocator or memory-pool callback,
 * in a latency-critical loop that cannot wait on the driver's allocator, or
 * next to a framework that owns all device memory.  (A host function
 * enqueued with cudaLaunchHostFunc may make no CUDA call, this one included:
 * call it from ordinary host code with the stream instead.)  The caller
 * passes everything as device pointers (the CSR list, the FP32 weights of
 * n_outputs outputs laid out [o * w_stride + j], the FP64 field and the
 * [n_outputs * n] output); the only scratch, the (hi, lo) split of the
 * field, is a fixed device array inside the library.
 * Limits: n <= DCPSE_NOALLOC_MAX_PARTICLES (larger n is rejected with
 * DCPSE_ERR_CAPACITY).  w_stride must be at least rowptr[n] (with one output
 * it may be 0); a smaller stride makes the weight streams overlap.
 * Set-up: the array (16 MiB) belongs to the library's device code, which the
 * CUDA runtime loads onto a GPU lazily, on the first call there; that call
 * also looks up the array's device address (cudaGetSymbolAddress).  So make
 * one call with n = 0 per device at start-up, before any callback or stream
 * capture: it does exactly that set-up and nothing else.  The array is then
 * held until the process exits; the cached address is stale after
 * cudaDeviceReset, so do not use this entry point after a reset.
 * All calls share the array: calls that overlap on the GPU (e.g. on two
 * streams) race and must be serialised by the caller.  Every output takes
 * the compensated FP32 sum; with w_stride equal to the list's entry count
 * the results equal dcpse_apply_batched(..., DCPSE_F32) of a plan
 * configured with DCPSE_APPLY_COMPENSATE_ALL and direct loading (mode 1)
 * bit for bit (the lanes per row follow from w_stride / n). */
#define DCPSE_NOALLOC_MAX_PARTICLES 2097152
int dcpse_apply_batched_f32_noalloc(int64_t n, int n_outputs, const int64_t* d_rowptr, const int32_t* d_cols,
                                    const float* d_w, int64_t w_stride, const double* d_f, double* d_out,
                                    void* stream);

/* ---- timing -------------------------------------------------------------
 * Optional CUDA-event timing of the plan's kernels on the plan's stream (the
 * role of the reference's std::chrono prints in Dcpse.cuh:581-716).
 * kernel ids: */
#define DCPSE_K_APPLY_BATCHED 0
#define DCPSE_K_SPLIT 1
#define DCPSE_K_ASSEMBLE 2
#define DCPSE_K_APPLY_TERM 3
#define DCPSE_K_NEIGHBORS 4
#define DCPSE_K_CORRECT 5 /* the FP64 correction pass of DCPSE_F32_BUDGET */
#define DCPSE_K_COUNT 6
int dcpse_plan_set_timing(dcpse_plan_t* plan, int enable);
/* Measured FP64 fused multiply-add throughput of the current GPU in TFLOP/s
 * (2 flops per FMA): the ceiling the FP64 assembly is reported against.
 * No counterpart in the reference. */
int dcpse_measure_fp64_peak(void* stream, double* tflops);
/* Apply schedule knobs (autotuning): lanes per row of the CSR kernels (0 =
 * from the mean row length, else 4/8/16/32) and the kernel (0 = automatic:
 * the sliced ELL kernel for DCPSE_F32 applies of whole operators, the direct
 * CSR kernel otherwise; 1 = CSR, direct loads; 2 = CSR, TMA-staged tiles;
 * 3 = CSR, direct loads in 8-deep batches; 4 = sliced ELL: the FP32 weights
 * in slices of 32 rows stored entry-major, rows sorted by length within
 * windows of 256, a row per thread; it keeps a second copy of the FP32
 * weights, built at assembly, and falls back to the CSR kernels when that
 * copy does not fit in device memory).  OR-ing DCPSE_APPLY_COMPENSATE_ALL
 * into the mode makes every output of the FP32 apply use the compensated sum
 * (by default only outputs with a term of order >= 2 do; the others take
 * plain fused sums). */
#define DCPSE_APPLY_COMPENSATE_ALL 16
/* The sliced kernels read their column and weight streams with the
 * streaming (evict-first) cache hint on a renumbered layout only (see
 * dcpse_plan_set_reorder); these bits force the hint on or off. */
#define DCPSE_APPLY_STREAM_HINT_ON 32
#define DCPSE_APPLY_STREAM_HINT_OFF 64
/* Scheduling of the sliced kernels.  Warp-scheduled: each warp takes the
 * next slice from a counter and stores its rows' outputs directly, so no
 * warp waits for the longest slice of its window.  Window-scheduled: a block
 * takes one window of 8 slices and its outputs leave in row order after the
 * window's barrier (always so for host-memory outputs and row chunks on
 * their own streams).  By default device-memory applies
 * are warp-scheduled when the window barrier would idle 15 % or more of the
 * warp time (slices of unequal length: graded clouds), measured when the
 * layout is built.  These bits force one schedule. */
#define DCPSE_APPLY_SLICE_WINDOWS 128
#define DCPSE_APPLY_SLICE_WARPS 256
int dcpse_plan_set_apply_config(dcpse_plan_t* plan, int lanes, int mode);
/* Assembly schedule knobs (autotuning): particles are processed in bins of
 * neighbour count of width bin_width (0 = index order; uneven clouds keep
 * warps of one CTA on similar work); the Gram and weight kernels run CTAs of
 * `warps` warps (2, 4 or 8); the QR kernel factorises each particle's
 * matrices with qr_lanes lanes (1, 2, 4, 8, 16 or 32; 0 = the fewest that
 * keep 6 warps per SM resident).  A lane count whose work space exceeds
 * shared memory makes dcpse_assemble return DCPSE_ERR_CAPACITY.  None of
 * these changes a result bit. */
int dcpse_plan_set_assembly_config(dcpse_plan_t* plan, int bin_width, int warps, int qr_lanes);
/* Synchronises the stream and reports DCPSE_ERR_TIMEOUT if a kernel's
 * bounded wait ran out since the plan was created. */
int dcpse_plan_check(dcpse_plan_t* plan);
/* Synchronises the stream; total device time and launches since the last reset. */
int dcpse_plan_timing(dcpse_plan_t* plan, int kernel, double* total_ms, int64_t* launches);
int dcpse_plan_reset_timing(dcpse_plan_t* plan);

#ifdef __cplusplus
}
#endif

#endif /* OPENFPM_DCPSE_CAPI_H */
