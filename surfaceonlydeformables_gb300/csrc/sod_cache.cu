// sod_cache.cu -- the reference's binary matrix files, so the original simulator can load matrices
// built here unchanged.
//
// Format of Eigen::save_matrix / load_matrix (include/matrix_io.hpp:14-61) for the reference's
// row-major dense matrices (include/type_declaration.hpp:18, 32): int64 rows, int64 cols, then
// rows x cols doubles in row-major order.  The time-domain cache of
// ElastodynamicsCQBEMMatrixCollection (src/elastodynamics_cqbem_matrix_collection.cpp:76-176) holds
// G_k.mat and H_k.mat (3V x 3V, H as computed: the reference negates it when loading, :140) and
// B_k.mat = [B_trans_k | B_euler_k] (3V x 6), k = 0..N.  The folder name is the caller's (the
// reference derives it from a hash of its JSON configuration, :41-52).
#include <cstdio>
#include <string>
#include <vector>

#include "sod_internal.h"

using namespace sod;

namespace {

constexpr size_t CHUNK = (size_t)64 << 20;  // bytes staged per device-to-host copy

// rows x cols row-major values (FP64 or FP32, host or device) -> FP64 row-major into `f`
int write_values(sod_context *ctx, FILE *f, const void *data, size_t n, int dtype, const std::string &path) {
    const size_t esz = dtype == SOD_F64 ? 8 : 4;
    const bool dev = ctx && is_device_pointer(data);
    std::vector<char> raw(dev ? std::min(CHUNK, n * esz) : 0);
    std::vector<double> conv(dtype == SOD_F32 ? std::min(CHUNK / esz, n) : 0);
    for (size_t e0 = 0; e0 < n; e0 += CHUNK / esz) {
        const size_t ne = std::min(CHUNK / esz, n - e0);
        const char *src = static_cast<const char *>(data) + e0 * esz;
        if (dev) {
            SOD_CHECK_CUDA(cudaMemcpyAsync(raw.data(), src, ne * esz, cudaMemcpyDeviceToHost, ctx->stream));
            SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
            src = raw.data();
        }
        const void *w = src;
        if (dtype == SOD_F32) {
            const float *s = reinterpret_cast<const float *>(src);
            for (size_t e = 0; e < ne; e++) conv[e] = (double)s[e];
            w = conv.data();
        }
        if (fwrite(w, sizeof(double), ne, f) != ne) {
            set_error("write failed: " + path);
            return SOD_ERR_INVALID_ARG;
        }
    }
    return SOD_OK;
}

int write_mat(sod_context *ctx, const std::string &path, const void *data, int64_t rows, int64_t cols, int dtype) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) {
        set_error("cannot open for writing: " + path);
        return SOD_ERR_INVALID_ARG;
    }
    const int64_t hdr[2] = {rows, cols};
    int rc = fwrite(hdr, sizeof(int64_t), 2, f) == 2 ? SOD_OK : SOD_ERR_INVALID_ARG;
    if (rc != SOD_OK) set_error("write failed: " + path);
    if (rc == SOD_OK) rc = write_values(ctx, f, data, (size_t)rows * (size_t)cols, dtype, path);
    if (fclose(f) != 0 && rc == SOD_OK) {
        set_error("write failed: " + path);
        rc = SOD_ERR_INVALID_ARG;
    }
    return rc;
}

}  // namespace

extern "C" {

int sod_mat_write(sod_context *ctx, const char *path, const void *data, int64_t rows, int64_t cols, int dtype) {
    SOD_REQUIRE(path && data, "null argument");
    SOD_REQUIRE(rows >= 0 && cols >= 0, "negative matrix size");
    SOD_REQUIRE(dtype == SOD_F64 || dtype == SOD_F32, "matrix dtype must be SOD_F64 or SOD_F32");
    if (ctx) SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    return write_mat(ctx, path, data, rows, cols, dtype);
}

int sod_mat_read(sod_context *ctx, const char *path, void *data, int64_t rows, int64_t cols) {
    SOD_REQUIRE(path && data, "null argument");
    SOD_REQUIRE(rows >= 0 && cols >= 0, "negative matrix size");
    if (ctx) SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    FILE *f = fopen(path, "rb");
    if (!f) {
        set_error(std::string("cannot open for reading: ") + path);
        return SOD_ERR_INVALID_ARG;
    }
    int64_t hdr[2] = {-1, -1};
    if (fread(hdr, sizeof(int64_t), 2, f) != 2 || hdr[0] != rows || hdr[1] != cols) {
        fclose(f);
        set_error(std::string("not a ") + std::to_string(rows) + " x " + std::to_string(cols) + " matrix file: " + path);
        return SOD_ERR_INVALID_ARG;
    }
    const size_t n = (size_t)rows * (size_t)cols;
    const bool dev = ctx && is_device_pointer(data);
    std::vector<double> buf(dev ? std::min(CHUNK / 8, n) : 0);
    for (size_t e0 = 0; e0 < n; e0 += CHUNK / 8) {
        const size_t ne = std::min(CHUNK / 8, n - e0);
        double *dst = dev ? buf.data() : static_cast<double *>(data) + e0;
        if (fread(dst, sizeof(double), ne, f) != ne) {
            fclose(f);
            set_error(std::string("truncated matrix file: ") + path);
            return SOD_ERR_INVALID_ARG;
        }
        if (dev) {
            cudaError_t e = cudaMemcpyAsync(static_cast<double *>(data) + e0, buf.data(), ne * 8,
                                            cudaMemcpyHostToDevice, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) fclose(f);
            SOD_CHECK_CUDA(e);
        }
    }
    fclose(f);
    return SOD_OK;
}

int sod_cqbem_write_cache(sod_context *ctx, const char *folder, int nV, int L, const void *G, const void *H,
                          const void *B_trans, const void *B_euler, int dtype) {
    SOD_REQUIRE(ctx && folder, "null argument");
    SOD_REQUIRE(nV >= 1 && L >= 1, "need nV >= 1 and L >= 1");
    SOD_REQUIRE(dtype == SOD_F64 || dtype == SOD_F32, "matrix dtype must be SOD_F64 or SOD_F32");
    SOD_REQUIRE((B_trans == nullptr) == (B_euler == nullptr), "B_trans and B_euler go together (B_k = [B_trans | B_euler])");
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const size_t esz = dtype == SOD_F64 ? 8 : 4;
    const int64_t n3 = 3LL * nV;
    const std::string dir(folder);
    for (int k = 0; k < L; k++) {
        if (G)
            SOD_TRY(write_mat(ctx, dir + "/G_" + std::to_string(k) + ".mat",
                              static_cast<const char *>(G) + (size_t)k * n3 * n3 * esz, n3, n3, dtype));
        if (H)
            SOD_TRY(write_mat(ctx, dir + "/H_" + std::to_string(k) + ".mat",
                              static_cast<const char *>(H) + (size_t)k * n3 * n3 * esz, n3, n3, dtype));
        if (B_trans) {
            // B_k = [B_trans_k | B_euler_k], 3V x 6 row-major
            std::vector<char> bt(n3 * 3 * esz), be(n3 * 3 * esz);
            const char *src[2] = {static_cast<const char *>(B_trans) + (size_t)k * n3 * 3 * esz,
                                  static_cast<const char *>(B_euler) + (size_t)k * n3 * 3 * esz};
            char *dstv[2] = {bt.data(), be.data()};
            for (int t = 0; t < 2; t++) {
                if (is_device_pointer(src[t])) {
                    SOD_CHECK_CUDA(cudaMemcpy(dstv[t], src[t], n3 * 3 * esz, cudaMemcpyDeviceToHost));
                } else {
                    std::copy(src[t], src[t] + n3 * 3 * esz, dstv[t]);
                }
            }
            std::vector<double> B(n3 * 6);
            for (int64_t r = 0; r < n3; r++)
                for (int c = 0; c < 6; c++) {
                    const char *p = (c < 3 ? bt.data() : be.data()) + (r * 3 + c % 3) * esz;
                    B[r * 6 + c] = dtype == SOD_F64 ? *reinterpret_cast<const double *>(p)
                                                     : (double)*reinterpret_cast<const float *>(p);
                }
            SOD_TRY(write_mat(ctx, dir + "/B_" + std::to_string(k) + ".mat", B.data(), n3, 6, SOD_F64));
        }
    }
    return SOD_OK;
}

}  // extern "C"
