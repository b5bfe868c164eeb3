// sod_internal.h -- host-side structures shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sod_gb300.h"
#include "sod_device.cuh"

namespace sod {

// ---- errors -------------------------------------------------------------------------------
void set_error(const std::string &msg);
struct Status {
    int code = SOD_OK;
};
#define SOD_CHECK_CUDA(expr)                                                                      \
    do {                                                                                          \
        cudaError_t _e = (expr);                                                                  \
        if (_e != cudaSuccess) {                                                                  \
            ::sod::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));               \
            return _e == cudaErrorMemoryAllocation ? SOD_ERR_OOM : SOD_ERR_CUDA;                 \
        }                                                                                         \
    } while (0)
#define SOD_REQUIRE(cond, msg)                                                                    \
    do {                                                                                          \
        if (!(cond)) {                                                                            \
            ::sod::set_error(msg);                                                                \
            return SOD_ERR_INVALID_ARG;                                                           \
        }                                                                                         \
    } while (0)
#define SOD_TRY(expr)                                                                             \
    do {                                                                                          \
        int _rc = (expr);                                                                         \
        if (_rc != SOD_OK) return _rc;                                                            \
    } while (0)

// ---- device buffer (owning) ---------------------------------------------------------------
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    int ensure(size_t n) {  // grow-only
        if (n <= bytes) return SOD_OK;
        release();
        if (n == 0) return SOD_OK;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
            return SOD_ERR_OOM;
        }
        bytes = n;
        return SOD_OK;
    }
    template <class T> T *as() const { return reinterpret_cast<T *>(p); }
};

// ---- quadrature point table passed by value to kernels ----------------------------------------
constexpr int MAX_TRI_PTS = 13 * 16;  // order-7 rule with subdivision 4
struct PointTable {
    int n;
    float4 p[MAX_TRI_PTS];  // (l0, l1, l2, w): barycentrics w.r.t. the whole face, weight / subdiv^2
};
struct PointD {
    double l0, l1, l2, w;
};
struct PointTableD {  // FP64 copy of the same table
    int n;
    PointD p[MAX_TRI_PTS];
};
struct GaussTable {  // 1-D Gauss-Legendre on [0,1] after subdivision: points and weights
    int n;
    double x[20], w[20];
};
int make_point_table(int order, int subdiv, PointTable &pt, PointTableD *ptd = nullptr);
int make_unit_gauss(int order, int subdiv, GaussTable &g);
const double (*tri_rule_table(int order, int &n))[4];
const double (*gl_rule_table(int order, int &n))[2];

// ---- context ------------------------------------------------------------------------------
}  // namespace sod

struct sod_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    std::atomic<int64_t> launches{0};
    int coll_threads = 0;  // 0 = automatic
    int gal_threads = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    // scratch
    sod::DevBuf sing;      // singular corrections
    sod::DevBuf sing_res;  // per-star-entry results of the double-float singular passes
    sod::DevBuf kconst;    // per-frequency constants
    sod::DevBuf staging;   // device staging for host outputs
    sod::DevBuf staging2;  // device staging for host inputs
    sod::DevBuf twiddle;   // inverse-transform twiddles
    sod::DevBuf freqbuf;   // Laplace-domain intermediates of the precompute
    sod::DevBuf small;     // small per-call tables (free terms, adjacency)
    sod::DevBuf gal_rows;  // Galerkin: unweighted rows of every test point (per frequency chunk)
    cudaStream_t copy_stream = nullptr;    // device-to-host copies overlapped with compute
    std::vector<cudaEvent_t> chunk_events;  // row-chunk completion markers (reused)
    sod::DevBuf gal_bsum;  // Galerkin: B_trans / B_angular sums of every test point
    sod::DevBuf gacc;      // collocation row accumulators in global memory (meshes too large for shared memory)
    sod::DevBuf dev_err;   // error word of the scatter kernels' bounded colour-phase waits (0 = none)
    bool wait_test = false;  // test hook: colour-phase barriers expect one arrival more than comes
    int precision = SOD_PRECISION_AUTO;  // regular-pass precision (sod_context_set_precision)
    void count(int n = 1) { launches += n; }
};

// After the context's stream is synchronised: SOD_ERR_TIMEOUT (and the word cleared) if a scatter
// kernel's bounded wait expired since the last check.
int take_device_error(sod_context *ctx);

struct sod_mesh {
    sod_context *ctx = nullptr;
    int nV = 0, nF = 0;
    bool has_vmap = false;
    std::vector<double> V, N;
    std::vector<int> F, vmap;
    // device copies
    sod::DevBuf dV, dN, dF, dVf, dCanon;
    // vertex stars: faces incident to each canonical vertex, with the singular corner
    std::vector<int> star_off, star_face, star_corner;
    sod::DevBuf dStarOff, dStarFace, dStarCorner;
    // per field vertex i: distinct vertices touched by its star faces (singular block slots)
    std::vector<int> nbr_off, nbr_vert, star_slot;  // star_slot: 3 slots per star entry
    sod::DevBuf dNbrOff, dNbrVert, dStarSlot;
    // colour-ordered face records for the deterministic scatter, keyed by threads-per-CTA
    struct Coloured {
        int ncolors = 0;
        std::vector<int> off;  // ncolors + 1
        sod::DevBuf dFaces;    // 4 float4 per face
        sod::DevBuf dCanonF;   // int4 per face (canonical corner ids) if vmap
        sod::DevBuf dOff;
    };
    std::map<int, std::unique_ptr<Coloured>> coloured;
    std::map<int, int> tuned;  // scatter CTA size chosen by the autotuner, key kind * 16 + fused B kinds
    // guards `coloured` and `tuned`: host threads sharing a mesh (a request loop's workers, or the
    // allocation-free entry point while another thread autotunes) may look up and insert at once;
    // recursive because the autotuners call coloured_for while they hold it
    mutable std::recursive_mutex sched_mu;
    // frequency-independent singular-quadrature geometry per (order, subdivision), double-float
    struct SingGeom {
        int nq2 = 0;          // points per star entry
        sod::DevBuf polar;    // [nq2][9][nstar] float2: r, rh.x, rh.y, rh.z, rh.n, w, w L0, w L1, w L2
        sod::DevBuf guig;     // [nq2][8][nstar] float2: r, rh.x, rh.y, rh.z, rh.n, w L_c J rho / r^2 (c = 0..2)
        sod::DevBuf guig_sub; // [9][nstar] double: Cauchy principal value subtraction (times kappa / 4 pi)
    };
    std::map<std::pair<int, int>, std::unique_ptr<SingGeom>> sing_geom;
    // Galerkin singular-pair entries per vertex and the two-ring slots of each row (sod_galerkin.cu)
    struct GalData {
        int nent = 0, nslots = 0, npairs = 0;
        sod::DevBuf ent, ent_off, slot_off, slot_vert;
        sod::DevBuf pairs;  // per distinct singular face pair: {f2, class}, j1, j2, {entry of test corner 0..2}
        // stars of the actual vertices (the support of each test function; with traction-discontinuity
        // splitting a split vertex owns only its own corners): faces in order, corner of the vertex
        sod::DevBuf astar_off, astar_face, astar_corner;
        int max_astar = 0;
    };
    std::unique_ptr<GalData> gal;
    int sing_geom_for(int sorder, int ssub, cudaStream_t stream, const SingGeom **out);
    // all faces in natural order (for the reduction kernels and Galerkin)
    sod::DevBuf dFacesNat, dCanonNat;
    int coloured_for(int threads, const Coloured **out);
};

namespace sod {
// Per-frequency constants travel as a __grid_constant__ kernel parameter (no host->device copy,
// no stream synchronisation); launches with more frequencies are split into chunks.
constexpr int MAX_FREQ_PER_LAUNCH = 40;
struct FreqTable {
    int n;
    KConst<float> kf[MAX_FREQ_PER_LAUNCH];
    KConst<double> kd[MAX_FREQ_PER_LAUNCH];
};
struct CollLaunch {
    const sod_mesh *mesh;
    int kind_mask;  // bit k set: assemble kind k (SOD_G .. SOD_B_ANGULAR)
    int nfreq;
    const KConst<double> *kc_host;  // host array, nfreq entries
    int order, subdiv, sorder, ssub, parts;
    void *out[4];  // device, per kind (null where the bit is clear)
    int out_dtype;
    long long freq_stride[4];  // elements between consecutive frequencies of out[kind]
    cudaStream_t stream;
    // collocation only: regular pass in compensated double-float arithmetic (sod_coll_compensated.cu)
    // instead of FP32; for time-domain outputs, whose late weights amplify FP32 noise by up to R^-N
    int compensated;
    // collocation only: host destinations of out[kind] (device staging).  When set, the scatter runs
    // in row chunks and each chunk's rows are copied to the host on the context's copy stream while
    // the next chunk computes; `stream` waits for the copies at the end.
    void *host[4];
};
int launch_collocation(sod_context *ctx, const CollLaunch &L);
// Galerkin assembly of G / H (sod_galerkin.cu); same launch description.
int launch_galerkin(sod_context *ctx, const CollLaunch &L);
// Singular passes in double-float (sod_singular.cu): fills the side buffers S[kind] (per kind in
// `mask`, layout of the regular kernels' epilogue) for nf frequencies; kc is a host array.
int launch_singular(sod_context *ctx, const sod_mesh *m, int mask, int sorder, int ssub, const KConst<double> *kc,
                    int nf, cd *const S[4], const long long S_fstride[4], cudaStream_t stream);
// Elastostatic (Kelvin) singular blocks of G / H into S (sod_singular.cu), FP64.
int launch_static_singular(sod_context *ctx, const sod_mesh *m, int mask, int sorder, int ssub, double nu, double mu,
                           cd *const S[4], cudaStream_t stream);
// Batched singular passes: one descriptor per object, flat work lists, launched by sod_batch.
struct SingBatchObj {
    int nV, nstar, nq2, pad0;
    const float2 *polar, *guig;
    const double *guig_sub;
    const int *star_off, *star_face, *star_slot, *nbr_off;
    const double *N;
    double2 *Rp, *Rg;  // per (frequency, component, star entry) results of the two passes
    cd *S[4];
    long long S_fstride[4];
    int kc_off, nf;
};
size_t sing_result_elems(int mask, int nstar, int nf, bool guiggiani);
// singular passes of a batch: `which` 0 polar (G, B_trans, B_angular), 1 Guiggiani (H), 2 combine
// of the kinds in `mask`; one CTA per item
int sing_batch_launch(sod_context *ctx, int which, int mask, const SingBatchObj *objs, const int4 *items, int nitems,
                      const KConst<double> *kcd, cudaStream_t stream);
// Compensated (double-float) regular collocation pass of one chunk of field vertices
// (sod_coll_compensated.cu); the CollArgs carry everything but the face schedule.
struct CollArgs;
int comp_scatter_threads(sod_context *ctx, sod_mesh *m, int kind, int *threads);
int launch_regular_compensated(sod_context *ctx, const sod_mesh *m, CollArgs a, int mask,
                               const sod_mesh::Coloured *colG, const sod_mesh::Coloured *colH, const int threads[2],
                               const PointTable &pt, const FreqTable &ft, int nvert, cudaStream_t stream);
// Assembly of the kinds in `mask` (sod_api.cu): the shared driver of the sod_cqbem_assemble* entry
// points, with the regular-pass precision chosen by the caller (compensated: time-domain outputs).
int assemble_kinds(sod_context *ctx, const sod_mesh *mesh, int mask, int method, double c1, double c2, double rho,
                   const double *s, int nfreq, int order, int subdiv, int sorder, int ssub, int parts,
                   void *const outs[4], int out_dtype, bool compensated);
// Allocation-free launcher over caller-provided scratch (see sod_collocation.cu).
int launch_collocation_prealloc(sod_context *ctx, const sod_mesh *m, int kind, double c1, double c2, double rho,
                                const double *s, int nfreq, int order, int subdiv, int sorder, int ssub, void *out,
                                int out_dtype, cd *scratch, long long scratch_elems, cudaStream_t stream);
bool is_device_pointer(const void *p);
// Batched persistent launches of the regular passes (sod_collocation.cu).  One BatchRegular holds
// the arguments of up to BATCH_OBJS objects in kernel-parameter space; `which` 2 G scatter (B kinds
// of the mask fused in), 3 H scatter, 4 B reduction.
constexpr int BATCH_OBJS = 112;
struct BatchRegular;
BatchRegular *batch_regular_new(int which, int mask, int threads, size_t smem, const PointTable &pt);
// scatter launch with the row accumulators in global memory (`slice` bytes per CTA); *rc reports
// allocation failures (the object is returned either way and must be freed)
constexpr int SCATTER_GLOBAL_THREADS = 256;
BatchRegular *batch_regular_new_global(sod_context *ctx, int which, int mask, size_t slice, int nitems_hint,
                                       const PointTable &pt, int *rc);
void batch_regular_free(BatchRegular *r);
int batch_regular_add(BatchRegular *r, const sod_mesh *m, int out_dtype, void *const out[4], cd *const S[4],
                      const sod_mesh::Coloured *col, int kc_off, int *slot);
int batch_regular_issue(sod_context *ctx, const BatchRegular *r, const int4 *items, int nitems, int *counter,
                        const KConst<float> *kcf, cudaStream_t stream);
// Dynamic shared memory and occupancy of the scatter variants (bm: B kinds fused into G).
size_t scatter_smem_bytes(int kind, int bm, int nV, int threads);
int scatter_occupancy(sod_context *ctx, int kind, int bm, bool batch, int threads, size_t smem, int *per_sm);
// Deterministic autotuner of the scatter kernels' CTA size (see sod_collocation.cu).
int autotune_scatter_threads(sod_context *ctx, sod_mesh *m, int kind, int bm, int *threads);
int launch_inverse_transform(sod_context *ctx, const void *Xhat, int in_dtype, int64_t M, int nfreq, int L,
                             double R, void *out, int out_dtype, cudaStream_t stream);
KConst<double> make_kconst(double c1, double c2, double rho, double sr, double si);
KConst<float> to_float(const KConst<double> &k);
// tensor-core (tcgen05) history convolution of a BF16 or FP32 bank (1 or 16 right-hand sides).  The plan
// holds the two TMA tensor maps (CUtensorMap, 128 bytes each), encoded once per bank.
struct HistTcPlan {
    alignas(64) unsigned char wmap[128];
    alignas(64) unsigned char xmap[128];
    int nrow = 0, ncol = 0, ldw = 0, K = 0, R = 0;
    const void *W = nullptr, *Xt = nullptr;
    bool f32 = false;  // FP32 bank (3xTF32) or BF16 bank
    bool ready = false;
};
size_t history_tc_partial_floats(int num_sms, int nrow, int R);
int history_tc_plan(HistTcPlan *plan, const void *W, const void *Xt, int nrow, int ncol, int ldw, int K, int R,
                    bool f32);
// err: device error word (first expired wait); err_mirror: pinned host word the finish kernel copies it to
int launch_history_tc(sod_context *ctx, const HistTcPlan *plan, const float *scale, int used, int head,
                      float *partial, const double *Bw, const double *A, double *out, int *err, int *err_mirror,
                      cudaStream_t stream);

// wavelet-compressed history weights (sod_wavelet.cu): Haar non-standard form of P W P^T per block
// b = 2 (k - 1) + {0: G, 1: -H}, top-(N^2 ratio) coefficients as CSR, merged for the per-step SpMV
struct WaveletBank;
int wavelet_bank_create(sod_context *ctx, int nV, int K, double ratio, WaveletBank **out);
void wavelet_bank_free(WaveletBank *w);
int wavelet_set_block(sod_context *ctx, WaveletBank *w, int b, const void *W, bool f64, double sign);
// ring slot `slot` <- wavelet vectors of p and u; aslot (6 doubles) <- a or zeros
int wavelet_push(sod_context *ctx, WaveletBank *w, const double *p, const double *u, const double *a, int slot,
                 double *aslot);
// out (3nV) = P^T reconstruct(sum over the `used` most recent steps); head = ring slot of the next push
int wavelet_convolve(sod_context *ctx, WaveletBank *w, int used, int head, double *out);
int64_t wavelet_bytes(const WaveletBank *w);
int wavelet_block(const WaveletBank *w, int b, int64_t *nnz, int *row_ptr, int *col, double *val, cudaStream_t st);
int wavelet_dims(const WaveletBank *w, int *N, int *L);

// One time step of several history banks in three launches (sod_history.cu), for the request loop:
// FP32 banks with one right-hand side on the CUDA-core engine, each bank at most once; p, u, b device
// vectors per bank.  A bank's b is bitwise the same as from sod_history_push + sod_history_convolve.
constexpr int HIST_GROUP_MAX = 48;
bool history_groupable(const sod_history *h);
int history_step_group(sod_context *ctx, sod_history *const *banks, int n, const double *const *p,
                       const double *const *u, double *const *b);

// dense LU solves (sod_solve.cu); X = A^-1 B, row-major device buffers, X may alias B
int solver_size(const sod_solver *s);
int solver_solve_device(sod_solver *s, int nrhs, const double *B, double *X);
// per-step form: GEMV with the kept inverse when there is one, else the LU solve (X must not alias B)
int solver_apply_device(sod_solver *s, int nrhs, const double *B, double *X);

}  // namespace sod
