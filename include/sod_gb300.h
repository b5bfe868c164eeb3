/*
 * sod_gb300.h -- C ABI of the GB300 (sm_103a) CQBEM precomputation library.
 *
 * Drop-in replacement for the BEM precomputation hot path of SurfaceOnlyDeformables:
 * Laplace-domain assembly of the elastodynamic CQBEM matrices G (single layer U), H (double
 * layer P), B_trans and B_angular by collocation or Galerkin quadrature, the FP64-accurate
 * inverse transform to convolution-quadrature time weights, the elastostatic Kelvin matrices
 * and the per-step history convolution.
 *
 * Conventions shared by every entry point
 *   - plain pointers and sizes; no C++ or framework types cross this boundary;
 *   - row-major layouts identical to the reference's Eigen row-major types
 *     (include/type_declaration.hpp:16-49 of the reference):
 *       V  double[nV][3]   vertex positions (already centred by the caller)
 *       F  int32 [nF][3]   triangle vertex indices, outward orientation
 *       N  double[nF][3]   unit face normals (NULL: computed from V, F)
 *       U, P              [3nV][3nV] complex (interleaved re, im)
 *       B_trans           [3nV][3]   complex
 *       B_angular         [3nV][3][3] complex ([row][j][k], the reference's ind_3d order)
 *   - output buffers are caller-owned and FULLY overwritten (there is no accumulate-into
 *     contract, unlike the reference's Galerkin kernels which add into a zeroed buffer);
 *   - a pointer may be host or device memory; the library detects which
 *     (cudaPointerGetAttributes) and copies host data through its own device buffers;
 *   - every call returns an int status (SOD_OK = 0); nothing prints, exits or aborts;
 *     sod_last_error() returns a thread-local message for the last failure;
 *   - results do not depend on thread count, launch configuration or batch composition:
 *     all reductions run in a fixed order (no floating-point atomics).
 *
 * The library needs an sm_103a GPU; without one every compute call returns
 * SOD_ERR_NO_DEVICE.  There is no CPU fallback.
 */
#ifndef SOD_GB300_H
#define SOD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
enum sod_status {
    SOD_OK = 0,
    SOD_ERR_INVALID_ARG = 1, /* bad size, order, kind, null pointer, degenerate input   */
    SOD_ERR_OOM = 2,         /* device or pinned-host allocation failed                 */
    SOD_ERR_CUDA = 3,        /* a CUDA runtime call failed                              */
    SOD_ERR_NO_DEVICE = 4,   /* no usable sm_103a device                                */
    SOD_ERR_TIMEOUT = 5,     /* a bounded device-side wait expired                      */
    SOD_ERR_UNSUPPORTED = 6, /* valid request outside the implemented envelope          */
    SOD_ERR_CAPACITY = 7     /* request exceeds an admission / footprint cap            */
};

/* ---- enumerations --------------------------------------------------------------------- */
enum sod_kind { SOD_G = 0, SOD_H = 1, SOD_B_TRANS = 2, SOD_B_ANGULAR = 3 };
enum sod_method { SOD_COLLOCATION = 0, SOD_GALERKIN = 1 };
enum sod_dtype { SOD_C128 = 0, SOD_C64 = 1, SOD_F64 = 2, SOD_F32 = 3, SOD_BF16 = 4 };
/* parts of an assembly to compute (for isolating the FP32 regular and FP64 singular passes) */
enum sod_parts { SOD_PART_REGULAR = 1, SOD_PART_SINGULAR = 2, SOD_PART_ALL = 3 };

typedef struct sod_context sod_context;
typedef struct sod_mesh sod_mesh;
typedef struct sod_batch sod_batch;

/* ---- library / diagnostics -------------------------------------------------------------- */
int sod_version(void);
const char *sod_last_error(void);
/* Host-side quadrature table, {l0,l1,l2,w} rows (w sums to 1), for order 1..5 (Cowper, as
 * include/integrator.hpp:55-113 of the reference) and 7 (13-point degree-7 rule, not in the
 * reference).  Returns the number of points via *npts.  Needs no GPU. */
int sod_triangle_rule(int order, double *out, int *npts);
/* CQ frequencies s_l = gamma(R zeta^l)/dt for l = 0..L/2, R = (1e-10)^(1/(2N)), L = N+1,
 * gamma_BDF1(z) = 1-z, gamma_BDF2(z) = 3/2 - 2z + z^2/2.  Replaces the prologue of
 * compute_G_matrices (src/elastodynamics_cqbem_G.cu:19-24,65).  s_out: (L/2+1) complex.
 * Needs no GPU. */
int sod_cq_frequencies(int bdf, double dt, int N, double *s_out, double *R_out, int *L_out);

/* ---- context: device, stream, scratch ----------------------------------------------------- */
int sod_context_create(int device, sod_context **ctx);
int sod_context_destroy(sod_context *ctx);
/* Work is issued on `stream` (a cudaStream_t; NULL = CUDA's default stream).  A new context uses
 * a non-blocking stream of its own.  A context's scratch buffers are reused call after call in
 * stream order, so one context must not be driven from two streams at once. */
int sod_context_set_stream(sod_context *ctx, void *stream);
/* Also reports SOD_ERR_TIMEOUT if a bounded device-side wait of a scatter kernel expired since the
 * last synchronising call (the results of that work are then not valid; the context stays usable). */
int sod_context_synchronize(sod_context *ctx);
/* Test hook for the timeout path: with stall != 0 the collocation scatter kernels of the per-call
 * assembly functions (sod_cqbem_assemble*) launched by this context initialise their colour-phase
 * barrier for one more arrival than ever comes, so every bounded wait runs out (about a second per
 * CTA wave) and the next synchronising call returns SOD_ERR_TIMEOUT.  Batched launches are not
 * affected.  0 (the default) restores normal operation. */
int sod_context_set_wait_test(sod_context *ctx, int stall);
/* Threads per CTA of the collocation scatter kernels (0 = automatic); for the autotuner. */
int sod_context_set_tuning(sod_context *ctx, int coll_threads, int galerkin_threads);
/* Precision of the regular (non-singular) collocation quadrature.  The geometry (distances,
 * directions, weights) is FP32 either way; FP32 evaluates the frequency-dependent terms (complex
 * exponentials, psi, kernel coefficients) and the sums in FP32 (~3e-7 relative error per
 * Laplace-domain matrix), COMPENSATED in double-float arithmetic on the FP32 pipes with
 * compensated sums (~3e-8, the FP32 geometry alone).  The inverse transform multiplies the late time
 * weights by up to R^-N = 1e5, so FP32 noise becomes ~1e-3 of the stacked time-domain weights, and
 * compensated evaluation brings them back to ~1e-7.  AUTO (the default): FP32 for the Laplace-domain
 * entry points (sod_cqbem_assemble*), COMPENSATED for time-domain outputs (sod_cqbem_precompute and
 * the request loop's assemblies).  FP32 / COMPENSATED force one for both.  The Galerkin regular pairs
 * and the batched kernels are FP32 in every mode.  No counterpart in the reference, whose regular
 * collocation G and B are FP32 and H FP64 (src/elastodynamics_cqbem_*_collocation.cu:15). */
enum sod_precision { SOD_PRECISION_AUTO = 0, SOD_PRECISION_FP32 = 1, SOD_PRECISION_COMPENSATED = 2 };
int sod_context_set_precision(sod_context *ctx, int precision);
/* Count of kernel launches issued by this context since creation (for launch accounting). */
int64_t sod_context_launch_count(const sod_context *ctx);

/* ---- mesh: device-resident geometry + precomputed topology -------------------------------- */
/* Uploads V, F (and N, or computes unit face normals), builds vertex stars, face colourings for
 * the deterministic scatter, and the singular-pair lists.  vmap: vertex_map_inverse of the
 * reference (NULL when traction discontinuity is off), nV entries in [0, nV).  Face indices outside
 * [0, nV), non-finite coordinates and zero-area faces are rejected with SOD_ERR_INVALID_ARG. */
int sod_mesh_create(sod_context *ctx, const double *V, int nV, const int *F, int nF, const double *N,
                    const int *vmap, sod_mesh **mesh);
int sod_mesh_destroy(sod_mesh *mesh);
/* The face colouring behind the deterministic scatter, on the host (no device needed): colour[f] for
 * every face such that no two faces of a colour share a vertex and no colour holds more than
 * `capacity` faces (the scatter CTA size: one round per colour, one face per thread); *ncolours
 * receives the colour count.  No reference counterpart (the reference adds with atomics). */
int sod_face_colouring(const int *F, int nF, int nV, int capacity, int *colour, int *ncolours);

/* ---- Laplace-domain assembly, one frequency (the drop-in kernels) ------------------------- */
/* Whole-matrix replacement of the reference's per-row / per-pair kernels for one Laplace
 * frequency s = (s_re, s_im):
 *   kind G, collocation : compute_elastodynamic_G_kernel_collocation over all rows
 *                         (src/elastodynamics_cqbem_G_collocation.cu:18-142; driver src/elastodynamics_cqbem_G.cu:122-146)
 *   kind H, collocation : src/elastodynamics_cqbem_H_collocation.cu:18-158 (src/elastodynamics_cqbem_H.cu:125-151)
 *   kind B_trans, coll. : src/elastodynamics_cqbem_B_trans_collocation.cu:17-124
 *   kind B_angular,coll.: src/elastodynamics_cqbem_B_angular_collocation.cu:17-143
 *   Galerkin (any kind) : non-singular pairs (..._galerkin_non_singular.cu) plus singular pairs
 *                         (src/elastodynamics_cqbem_galerkin_singular.cpp), i.e. the sum formed at
 *                         src/elastodynamics_cqbem_G.cu:67-120.
 * Regular integrals run in FP32, singular ones in FP64.  order: triangle rule (1..5, 7);
 * subdiv: uniform subdivision (1..4); sorder/ssub: 1-D Gauss order (1..5) and subdivision of the
 * singular rules (the reference uses order/subdiv for both).
 * out: complex, dtype SOD_C128 (reference layout) or SOD_C64; shape per kind as above. */
int sod_cqbem_assemble(sod_context *ctx, const sod_mesh *mesh, int kind, int method, double c1, double c2,
                       double rho, double s_re, double s_im, int order, int subdiv, int sorder, int ssub,
                       int parts, void *out, int out_dtype);

/* Same for nfreq frequencies s[2*l], s[2*l+1] in one launch; out holds nfreq consecutive matrices.
 * Replaces the frequency loop of compute_{G,H,B_trans,B_angular}_matrices
 * (src/elastodynamics_cqbem_G.cu:63-151 and its H / B_trans / B_angular twins). */
int sod_cqbem_assemble_frequencies(sod_context *ctx, const sod_mesh *mesh, int kind, int method, double c1,
                                   double c2, double rho, const double *s, int nfreq, int order, int subdiv,
                                   int sorder, int ssub, int parts, void *out, int out_dtype);

/* Every kind whose output pointer is non-NULL, for nfreq frequencies, in one call: the kinds share
 * the FP64 radial terms of the polar-rule singular pass (G, B_trans, B_angular) and the regular
 * B_trans/B_angular pass.  The per-object unit of compute_H_matrices + compute_G_matrices +
 * compute_B_trans_matrices + compute_B_angular_tensors (src/elastodynamics_cqbem_matrix_collection.cpp:90-93,165-166). */
int sod_cqbem_assemble_all(sod_context *ctx, const sod_mesh *mesh, int method, double c1, double c2, double rho,
                           const double *s, int nfreq, int order, int subdiv, int sorder, int ssub, int parts,
                           void *out_G, void *out_H, void *out_B_trans, void *out_B_angular, int out_dtype);

/* Allocation-free variant of sod_cqbem_assemble_frequencies (collocation, one kind).  It has no
 * counterpart in the reference.  It is for callers that cannot allocate device memory while they
 * run -- a host program that reserves its whole device memory budget at start-up and forbids
 * libraries from calling the CUDA allocator, or a real-time step loop in which cudaMalloc (which
 * may synchronise the device) would break the frame budget.  The call makes no cudaMalloc /
 * cudaFree or other allocation: its only scratch, the FP64 singular side buffer, is a fixed 4 MiB
 * device array inside the library (held on every GPU that loads the library until exit).
 * Requirements and limits:
 *   - `out` must be device memory; `mesh` must have been assembled once through
 *     sod_cqbem_assemble* during set-up (that builds the scatter schedule, with allocation);
 *   - one frequency's side buffer (9 complex doubles per neighbour slot for G/H, 9 or 27 per vertex
 *     for B_trans/B_angular) must fit in 4 MiB, else SOD_ERR_CAPACITY; frequencies are processed
 *     in chunks that fit;
 *   - the G/H row block must also fit in shared memory (48 bytes per vertex for G, 72 for H; there
 *     is no global-memory accumulator here), else SOD_ERR_CAPACITY.  Together: G up to about 4100
 *     vertices (the scratch), H up to about 3200 (shared memory);
 *   - the first call on a device looks up the array's device address (cudaGetSymbolAddress); make
 *     that first call before any stream capture;
 *   - all calls share the array: calls whose kernels overlap on the GPU (other streams, other host
 *     threads) race on it and must be serialised by the caller. */
int sod_cqbem_assemble_noalloc(sod_context *ctx, const sod_mesh *mesh, int kind, double c1, double c2, double rho,
                               const double *s, int nfreq, int order, int subdiv, int sorder, int ssub, void *out,
                               int out_dtype);

/* ---- batched assembly of many objects (persistent kernels under a CUDA graph) ------------------- */
/* The reference assembles one object at a time, one launch per frequency
 * (ElastodynamicsCQBEMMatrixCollection::init per object group, src/simulator.cpp:102,118).  A batch
 * takes every frequency of every object into persistent launches fed from an (object, field
 * vertex, frequency) work queue, largest objects first, and replays them as one CUDA graph.
 * kind_mask: bit k selects kind k for every object of the batch.  Outputs: device memory, one
 * buffer per (object, kind) holding nfreq consecutive matrices in the reference layout.  An
 * object's results are identical whether it is run alone or in a batch. */
int sod_batch_create(sod_context *ctx, int kind_mask, int out_dtype, sod_batch **batch);
int sod_batch_add(sod_batch *batch, const sod_mesh *mesh, double c1, double c2, double rho, const double *s,
                  int nfreq, int order, int subdiv, int sorder, int ssub, void *out_G, void *out_H,
                  void *out_B_trans, void *out_B_angular);
/* Builds descriptors, colourings, work lists and captures the graph (allocates; call at set-up). */
int sod_batch_finalize(sod_batch *batch);
/* Replays the graph on the context's stream (finalizes first if needed). */
int sod_batch_run(sod_batch *batch);
/* Number of persistent launches in one replay. */
int sod_batch_launch_count(const sod_batch *batch);
/* Runs the step's launches one by one on the context's stream with CUDA events between them and
 * returns, per launch: which pass (0 weakly singular, 1 Guiggiani, 2 G scatter, 3 H scatter,
 * 4 B reduction, 5 singular combine of G/B_trans/B_angular, 6 singular combine of H), its work
 * (kernel evaluations; singular quadrature points for 0/1; vertex-frequencies for 5/6) and its
 * device time in ms.  Arrays hold `cap` >= sod_batch_launch_count() entries.  Synchronises the stream. */
int sod_batch_profile(sod_batch *batch, int cap, int *which, double *evals, float *ms);
int sod_batch_destroy(sod_batch *batch);

/* ---- elastostatic BEM matrices ----------------------------------------------------------------- */
/* Replaces ElasticsBEMMatrixCollection::compute_elastostatic_{G,H}_matrix_{collocation,galerkin}
 * (src/elastics_bem_matrix_collection.cpp:43-385): the Kelvin single- and double-layer matrices,
 * 3nV x 3nV row-major, H with the rigid-mode diagonal correction H_ii = -sum_{j != i} H_ij (Galerkin
 * H also with the mass matrix C added first, as the reference does).  Regular faces / face pairs in
 * FP32, singular ones and the correction in FP64 (double-float Sauter-Schwab pairs for Galerkin;
 * the reference integrates those with the regular order: pass sorder = order, ssub = subdiv for
 * parity).  out: SOD_F64 or SOD_F32, host or device.  method: SOD_COLLOCATION or SOD_GALERKIN. */
int sod_elastostatic_assemble(sod_context *ctx, const sod_mesh *mesh, int kind, int method, double nu, double mu,
                              int order, int subdiv, int sorder, int ssub, void *out, int out_dtype);

/* ---- per-step history convolution ----------------------------------------------------------- */
/* Replaces the dense history loop of ElastodynamicsCQBEMObject::estimate_next_state
 * (src/elastodynamics_cqbem_object.cpp:44-48):
 *   b = sum_{i=0}^{min(n,K)-1} G_{i+1} p_{n-1-i} - H_{i+1} u_{n-1-i} + B_{i+1} a_{n-1-i}
 * (H as computed by the CQ precompute, i.e. before the reference's negation at load,
 * src/elastodynamics_cqbem_matrix_collection.cpp:140).  A bank keeps G_k, -H_k (nrow x ncol each,
 * k = 1..K) device-resident as FP32 or as BF16 with one FP32 scale per (k, matrix, row), B_k
 * (nrow x 6, FP64) and a ring of the last K steps' vectors.  R right-hand sides per step (1 or 16);
 * vectors are [ncol][R] row-major doubles, a is [6][R], b is [nrow][R].  Host or device pointers. */
typedef struct sod_history sod_history;
int sod_history_create(sod_context *ctx, int nrow, int ncol, int K, int R, int weight_dtype, sod_history **bank);
/* G_k, H_k: nrow x ncol row-major, dtype SOD_F64 or SOD_F32; k in 1..K. */
int sod_history_set_weights(sod_history *bank, int k, const void *G_k, const void *H_k, int in_dtype);
int sod_history_set_b(sod_history *bank, int k, const double *B_k);
/* Appends step n's p, u (and a, may be NULL) to the ring. */
int sod_history_push(sod_history *bank, const double *p, const double *u, const double *a);
/* b for the next step from the pushed history (the min(n, K) most recent steps). */
int sod_history_convolve(sod_history *bank, double *b);
int sod_history_reset(sod_history *bank);
/* Engine for the convolution: AUTO (tensor cores for BF16 banks and for FP32 banks with R = 16,
 * CUDA cores for FP32 banks with R = 1), CUDA_CORES, or TENSOR_CORES.  FP32 banks on the tensor
 * cores use a 3xTF32 split (FP32 accuracy).  A change of engine empties the history ring (the
 * engines keep it in different layouts). */
enum { SOD_HISTORY_ENGINE_AUTO = 0, SOD_HISTORY_ENGINE_CUDA_CORES = 1, SOD_HISTORY_ENGINE_TENSOR_CORES = 2 };
int sod_history_set_engine(sod_history *bank, int engine);
/* Wavelet-compressed bank: replaces CompressedMatrix<1> / CompressedVector<1> of the compressed
 * history (include/wavelets.hpp:337-436, src/elastodynamics_cqbem_object.cpp:31-41, 217-226,
 * src/elastodynamics_cqbem_matrix_collection.cpp:95-131).  Square 3nV x 3nV weights, one right-hand
 * side.  sod_history_set_weights then permutes each matrix (dof i -> i / 3 + (i % 3) nV), takes the
 * non-standard Haar decomposition of the zero-padded matrix (size Np = 2^ceil(log2 3nV); FP64,
 * bit-identical to a plain FP64 evaluation in the reference's order) and keeps the (int)(9 nV^2 ratio)
 * coefficients of largest magnitude (all nonzero ones if that is 0; ties at the threshold in (row,
 * column) order).  push, convolve, reset and the B terms work as for a dense bank; the per-step
 * product is one sparse pass over all kept coefficients plus the inverse transform.  3nV <= 16384.
 * sod_history_bytes reports the kept coefficients (12 bytes each). */
int sod_history_create_compressed(sod_context *ctx, int nV, int K, double ratio, sod_history **bank);
/* Kept coefficients of G_k (which = 0) or -H_k (which = 1) as CSR of the (2Np - 2)^2 matrix (columns
 * ascending; row_ptr has 2Np - 1 entries).  Pass NULL arrays to get nnz only.  Host arrays. */
int sod_history_compressed_matrix(sod_history *bank, int k, int which, int64_t *nnz, int32_t *row_ptr,
                                  int32_t *col, double *val);
/* The same matrix as the reference's .cpmat file (save_compressed_matrix, include/wavelets.hpp:474-502),
 * so the original simulator loads it unchanged (its cache names are H_k_<ratio>.cpmat / G_k_<ratio>.cpmat). */
int sod_history_write_cpmat(sod_history *bank, int k, int which, const char *path);
int sod_history_bytes(const sod_history *bank, int64_t *weight_bytes);
int sod_history_destroy(sod_history *bank);

/* ---- dense solves downstream of the assembly ------------------------------------------------- */
/* Replace the Eigen::PartialPivLU uses of ElastodynamicsCQBEMMatrixCollection::init
 * (src/elastodynamics_cqbem_matrix_collection.cpp:200-214: H_inv.compute(H_0), u_p = H_inv.solve(G'),
 * H_inv_B_trans / H_inv_B_euler, H_inv.inverse()) and the per-step H_inv.solve(b)
 * (src/elastodynamics_cqbem_object.cpp:63): LU with partial pivoting in FP64 on the device (this
 * library's blocked right-looking factorisation, LAPACK's pivot choice).  All matrices are row-major
 * FP64, host or device.  A singular matrix gives SOD_ERR_INVALID_ARG. */
typedef struct sod_solver sod_solver;
int sod_solver_create(sod_context *ctx, int n, const double *A, sod_solver **solver);
/* X = A^-1 B, B and X n x nrhs (X may alias B). */
int sod_solver_solve(sod_solver *solver, int nrhs, const double *B, double *X);
/* A^-1, n x n. */
int sod_solver_inverse(sod_solver *solver, double *Ainv);
/* Keeps A^-1 on the device (n^2 doubles), as the reference's H_inv.inverse(): the per-step
 * sod_history_convolve_solve then applies it as one FP64 GEMV instead of two triangular solves. */
int sod_solver_keep_inverse(sod_solver *solver);
int sod_solver_destroy(sod_solver *solver);
/* One served time step on the device: u = A^-1 b with b = sod_history_convolve's result ([nrow][R]);
 * the solver's n must equal the bank's nrow. */
int sod_history_convolve_solve(sod_history *bank, sod_solver *solver, double *u);

/* Replace the Eigen::CompleteOrthogonalDecomposition objects B_trans_inv / B_euler_inv
 * (include/elastodynamics_cqbem_matrix_collection.hpp:43, src/elastodynamics_cqbem_matrix_collection.cpp:
 * 184-191: B_trans_inv.solve(H), .solve(G'), B_euler_inv.solve(B_trans), ...): the minimum-norm
 * least-squares solution X = B^+ Y of a tall B (m x k, m >= k, 1 <= k <= 8; 3V x 3 in the reference).
 * Column-pivoted Householder QR, numerical rank by Eigen's default threshold
 * (|R_ii| > eps * k * max |R_ii|), and for a rank-deficient B the complete orthogonal decomposition.
 * FP64 on the device; B, Y (m x ncols) and X (k x ncols) row-major, host or device. */
typedef struct sod_lstsq sod_lstsq;
int sod_lstsq_create(sod_context *ctx, int m, int k, const double *B, sod_lstsq **lstsq);
int sod_lstsq_rank(const sod_lstsq *lstsq, int *rank);
int sod_lstsq_solve(sod_lstsq *lstsq, int ncols, const double *Y, double *X);
/* B^+ itself, k x m. */
int sod_lstsq_pinv(sod_lstsq *lstsq, double *P);
int sod_lstsq_destroy(sod_lstsq *lstsq);

/* Replaces the u_p computation of ElastostaticsBEMMatrixCollection::init
 * (src/elastostatics_bem_matrix_collection.cpp:58-89): with H, G the elastostatic matrices of
 * sod_elastostatic_assemble (3nV x 3nV row-major FP64, host or device) and T the area-weighted
 * rigid modes of the mesh,
 *   u_p = (H^T H + (tr H / 3nV)^2 T^T T)^-1 H^T G (I - T^T (T T^T)^-1 T).
 * The symmetric positive definite system is factored by Cholesky (the reference's LDL^T); FP64 on
 * the device with this library's GEMM and Cholesky kernels.  u_p: 3nV x 3nV row-major, host or device.
 * SOD_ERR_INVALID_ARG if the regularised matrix is not positive definite. */
int sod_elastostatic_u_p(sod_context *ctx, const sod_mesh *mesh, const double *H, const double *G, double *u_p);
/* T (6 x 3nV row-major, host or device): rows 0-2 translations (A_e / 6 per face corner), rows 3-5
 * rotations (A_e / 24 [v_0 + v_1 + v_2 + v_i]_x), A_e the doubled face area
 * (src/elastostatics_bem_matrix_collection.cpp:61-79). */
int sod_elastostatic_rigid_modes(sod_context *ctx, const sod_mesh *mesh, double *T);

/* ---- the reference's matrix files ------------------------------------------------------------ */
/* Eigen::save_matrix / load_matrix format (include/matrix_io.hpp:14-61): int64 rows, int64 cols,
 * then the row-major doubles.  data: host or device, SOD_F64 or SOD_F32 (written as doubles).
 * sod_mat_read reads into FP64 (host or device) and checks the dimensions.  ctx may be NULL when
 * data is host memory. */
int sod_mat_write(sod_context *ctx, const char *path, const void *data, int64_t rows, int64_t cols, int dtype);
int sod_mat_read(sod_context *ctx, const char *path, void *data, int64_t rows, int64_t cols);
/* The time-domain cache of ElastodynamicsCQBEMMatrixCollection::init
 * (src/elastodynamics_cqbem_matrix_collection.cpp:76-176) in `folder`: G_k.mat, H_k.mat (3V x 3V,
 * H as computed, before the reference's negation at load) and B_k.mat = [B_trans_k | B_euler_k]
 * (3V x 6), k = 0..L-1, from sod_cqbem_precompute's outputs ([L][...], host or device, SOD_F64 or
 * SOD_F32).  Any of G, H, (B_trans, B_euler) may be NULL.  The folder must exist. */
int sod_cqbem_write_cache(sod_context *ctx, const char *folder, int nV, int L, const void *G, const void *H,
                          const void *B_trans, const void *B_euler, int dtype);

/* ---- request loop (continuous batching) ------------------------------------------------------ */
/* A server owns `slots` assembly contexts and one step context on `device`.  Assembly requests
 * build a resident object (CQ precompute of G_k, H_k, k = 1..N, into an FP32 history bank, BDF
 * order bdf, collocation with the 2D rule `order` and subdivision `subdiv`); the request id is the
 * object id.  Step requests push p, u (3nV doubles each) of that object and produce
 * b = sum_k G_k p_{n-k} - H_k u_{n-k} (3nV doubles, read with sod_server_result).  Requests are
 * admitted while slots are free and the bytes of resident banks plus in-flight assembly buffers
 * stay below hbm_cap_bytes (least recently used idle objects are evicted; later steps for them
 * complete with SOD_ERR_INVALID_ARG).  All calls are thread-safe. */
typedef struct sod_server sod_server;
int sod_server_create(int device, int64_t hbm_cap_bytes, int slots, int max_vertices, sod_server **server);
int sod_server_submit_assembly(sod_server *server, const double *V, int nV, const int *F, int nF, double E,
                               double nu, double rho, int bdf, double dt, int N, int order, int subdiv,
                               int64_t *request_id);
int sod_server_submit_step(sod_server *server, int64_t object_id, const double *p, const double *u, int n,
                           int64_t *request_id);
/* Up to `cap` completions since the last call: request ids, status codes, latency (ns, submission to
 * completion). */
int sod_server_poll(sod_server *server, int64_t *ids, int *status, int64_t *latency_ns, int cap, int *n);
int sod_server_result(sod_server *server, int64_t request_id, double *b, int n);
/* Waits until every submitted request has completed (SOD_ERR_TIMEOUT after timeout_s seconds). */
int sod_server_drain(sod_server *server, double timeout_s);
int sod_server_stats(sod_server *server, int64_t *committed_bytes, int *resident_objects);
int sod_server_destroy(sod_server *server);

/* ---- time-domain precomputation of one object ------------------------------------------------ */
/* Replaces compute_H_matrices, compute_G_matrices, compute_B_trans_matrices,
 * compute_B_angular_tensors and compute_B_euler_matrices of ElastodynamicsCQBEMMatrixCollection
 * (src/elastodynamics_cqbem_{G,H,B_trans,B_angular}.cu, src/elastodynamics_cqbem_matrix_collection.cpp:90-93,
 * 165-167, 280-305).  CQ frequencies from (bdf, dt, N), L = N+1 time weights per kind:
 *   G_out  [L][3nV][3nV], H_out [L][3nV][3nV] (H_0 includes the free term C; not negated),
 *   B_trans_out [L][3nV][3], B_angular_out [L][3nV][3][3] (with the B_trans (x - cm) shift),
 *   B_euler_out [L][3nV][3].
 * Any output may be NULL; all non-NULL outputs must be device memory; dtype SOD_F64 or SOD_F32.
 * nu is the Poisson ratio (collocation free term); cm the centre of mass (3 doubles). */
int sod_cqbem_precompute(sod_context *ctx, const sod_mesh *mesh, int method, double c1, double c2, double rho,
                         double nu, int bdf, double dt, int N, int order, int subdiv, int sorder, int ssub,
                         const double *cm, void *G_out, void *H_out, void *B_trans_out, void *B_angular_out,
                         void *B_euler_out, int out_dtype);

/* ---- inverse transform to CQ time weights (FP64-accurate) --------------------------------- */
/* X_n = R^-n / L * sum_{l=0}^{L/2} c_l Re(Xhat_l zeta^-nl),  c_0 = 1, c_l = 2 otherwise except
 * c_{L/2} = 1 for even L;  n = 0..L-1 (src/elastodynamics_cqbem_G.cu:166-179).
 * Xhat: nfreq = L/2+1 blocks of M complex (dtype SOD_C128 or SOD_C64), out: L blocks of M reals
 * (SOD_F64 or SOD_F32).  SOD_F64 output accumulates in FP64 (agrees with an FP64 CPU transform to
 * <= 1e-10 of the stacked Frobenius norm); SOD_F32 output uses double-float arithmetic on the FP32
 * pipes (about 2^-48 of the term magnitude before the final FP32 rounding). */
int sod_cq_inverse_transform(sod_context *ctx, const void *Xhat, int in_dtype, int64_t M, int nfreq, int L,
                             double R, void *out, int out_dtype);

#ifdef __cplusplus
}
#endif
#endif /* SOD_GB300_H */
