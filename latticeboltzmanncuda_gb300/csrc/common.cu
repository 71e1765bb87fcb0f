// Shared helpers: error reporting, device allocation accounting, deterministic reduction finaliser.
#include <cstdio>

#include "lbm_internal.h"

namespace lbm {

namespace {
thread_local std::string g_thread_error;

// out[k] (+)= sum over b of partials[b*ncomp + k] (ncomp <= FIN_MAX): thread t sums the blocks t,
// t + FIN_THREADS, ... in that order, then a fixed tree over the threads -- the same order on every
// run, with the loads of many blocks in flight at once.
constexpr int FIN_THREADS = 256, FIN_MAX = 4;

__global__ void __launch_bounds__(FIN_THREADS) finalize_kernel(const double *__restrict__ partials, int nblocks,
                                                               int ncomp, double *out, int accumulate, double *also) {
    __shared__ double sm[FIN_MAX][FIN_THREADS];
    const int t = threadIdx.x;
    for (int k = 0; k < ncomp; ++k) {
        double s = 0.0;
        for (int b = t; b < nblocks; b += FIN_THREADS) s += partials[(int64_t)b * ncomp + k];
        sm[k][t] = s;
    }
    __syncthreads();
    for (int h = FIN_THREADS / 2; h > 0; h >>= 1) {
        if (t < h)
            for (int k = 0; k < ncomp; ++k) sm[k][t] += sm[k][t + h];
        __syncthreads();
    }
    if (t < ncomp) {
        const double v = accumulate ? out[t] + sm[t][0] : sm[t][0];
        out[t] = v;
        if (also) also[t] = v;
    }
}
}  // namespace

const char *thread_error() { return g_thread_error.c_str(); }

lbm_status set_thread_error(lbm_status s, const std::string &msg) {
    g_thread_error = msg;
    return s;
}

lbm_status fail(lbm_ctx *ctx, lbm_status s, const std::string &msg) {
    if (ctx) ctx->err = msg;
    g_thread_error = msg;
    return s;
}

lbm_status cuda_fail(lbm_ctx *ctx, cudaError_t e, const char *what) {
    std::string msg = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(ctx, e == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA, msg);
}

lbm_status dalloc(lbm_ctx *ctx, void **p, size_t bytes, const char *what) {
    *p = nullptr;
    if (bytes == 0) return LBM_OK;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(ctx, LBM_ERR_OOM,
                    std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes for " + what + " failed: " +
                        cudaGetErrorString(e));
    }
    ctx->device_bytes += bytes;
    return LBM_OK;
}

void dfree(lbm_ctx *ctx, void *p, size_t bytes) {
    if (!p) return;
    cudaFree(p);
    ctx->device_bytes -= bytes;
}

lbm_status ensure_scratch(lbm_ctx *ctx, size_t n) {
    if (ctx->scratch.n >= n) return LBM_OK;
    dfree(ctx, ctx->scratch.partials, ctx->scratch.n * sizeof(double));
    ctx->scratch.partials = nullptr;
    ctx->scratch.n = 0;
    void *p = nullptr;
    lbm_status s = dalloc(ctx, &p, n * sizeof(double), "reduction scratch");
    if (s != LBM_OK) return s;
    ctx->scratch.partials = static_cast<double *>(p);
    ctx->scratch.n = n;
    return LBM_OK;
}

cudaError_t finalize_sums(cudaStream_t s, const double *partials, int nblocks, int ncomp, double *out,
                          bool accumulate, double *also) {
    if (ncomp < 1 || ncomp > FIN_MAX) return cudaErrorInvalidValue;
    finalize_kernel<<<1, FIN_THREADS, 0, s>>>(partials, nblocks, ncomp, out, accumulate ? 1 : 0, also);
    return cudaGetLastError();
}

}  // namespace lbm
