// sod_noalloc.cu -- an assembly entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc while they run: a simulator that reserves its whole device
// memory budget up front and forbids libraries from touching the CUDA allocator, or a real-time
// step loop in which a cudaMalloc (which may synchronise the device) would break the frame budget.
// sod_cqbem_assemble_noalloc serves them.  The only scratch the collocation assembly needs -- the
// FP64 side buffer that carries the singular-face integrals to the regular pass -- lives in the
// file-scope device array below, so the call itself performs no allocation of any kind; the caller
// passes the inputs (a mesh created during set-up) and a device output buffer.
//
// The array occupies SOD_NOALLOC_SCRATCH_BYTES on every GPU that loads the library, until exit.
// Every call shares it: two calls whose kernels overlap on the GPU (different streams, or
// different host threads) race on it and must be serialised by the caller.  It keeps the contents
// of the last call; nothing in it has to start at zero, because the singular pass writes every slot
// of the side buffer before the regular pass reads it.
#include <mutex>

#include "sod_internal.h"

namespace sod {

constexpr long long SOD_NOALLOC_SCRATCH_BYTES = 4LL << 20;  // 4 MiB
static __device__ __align__(256) cd g_noalloc_scratch[SOD_NOALLOC_SCRATCH_BYTES / sizeof(cd)];

// Host code must not use g_noalloc_scratch as an address (it is a host-side stand-in); the device
// address is looked up once per device, with that device current, and cached.
static cd *g_scratch_addr[64];
static std::mutex g_scratch_mu;

static int noalloc_scratch(int device, cd **out) {
    SOD_REQUIRE(device >= 0 && device < 64, "device index out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[device]) {
        SOD_CHECK_CUDA(cudaSetDevice(device));
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            set_error(std::string("cudaGetSymbolAddress(noalloc scratch): ") + cudaGetErrorString(e));
            return SOD_ERR_CUDA;
        }
        g_scratch_addr[device] = static_cast<cd *>(p);
    }
    *out = g_scratch_addr[device];
    return SOD_OK;
}

}  // namespace sod

using namespace sod;

extern "C" int sod_cqbem_assemble_noalloc(sod_context *ctx, const sod_mesh *mesh, int kind, double c1, double c2,
                                          double rho, const double *s, int nfreq, int order, int subdiv, int sorder,
                                          int ssub, void *out, int out_dtype) {
    SOD_REQUIRE(ctx != nullptr, "null context");
    SOD_REQUIRE(mesh && mesh->ctx == ctx, "mesh does not belong to this context");
    SOD_REQUIRE(out_dtype == SOD_C128 || out_dtype == SOD_C64, "output dtype must be complex128 or complex64");
    SOD_REQUIRE(s != nullptr && nfreq >= 1 && nfreq <= 65535, "need 1..65535 Laplace frequencies");
    SOD_REQUIRE(c1 > 0 && c2 > 0 && rho > 0 && std::isfinite(c1) && std::isfinite(c2) && std::isfinite(rho),
                "wave speeds and density must be positive and finite");
    for (int l = 0; l < nfreq; l++)
        SOD_REQUIRE(std::isfinite(s[2 * l]) && std::isfinite(s[2 * l + 1]) && (s[2 * l] != 0.0 || s[2 * l + 1] != 0.0),
                    "Laplace frequencies must be finite and non-zero");
    SOD_REQUIRE(out != nullptr && is_device_pointer(out), "the allocation-free entry point needs a device output buffer");
    cd *scratch = nullptr;
    SOD_TRY(noalloc_scratch(ctx->device, &scratch));
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    return launch_collocation_prealloc(ctx, mesh, kind, c1, c2, rho, s, nfreq, order, subdiv, sorder, ssub, out,
                                       out_dtype, scratch, SOD_NOALLOC_SCRATCH_BYTES / (long long)sizeof(cd),
                                       ctx->stream);
}
