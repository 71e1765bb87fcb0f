// Allocation-free D2Q9 conservation sums (lbm_d2q9_conservation_noalloc).
//
// Some callers cannot allocate device memory while they run: an application that hands the
// solver a fixed device-memory budget and accounts for every byte of it (an embedding framework
// that owns all device memory, or the admission budget of a request-serving loop), and loops with
// a latency bound, where a cudaMalloc/cudaFree would synchronise the device and stall the work
// queued on other streams.  This entry point is the conservation reduction for them: the caller
// passes the populations, the flags and the output buffer, all in device memory it owns, and the
// per-block partial sums go to a fixed array that the library holds in device memory.
//
// The array is a file-scope static __device__ array of LBM_NOALLOC_MAX_ROWS / 4 partial triples
// (192 KiB); every GPU that loads the library holds it until the process exits.  Host code reaches
// it through the address that cudaGetSymbolAddress returns for the current CUDA context, looked up
// on the first call made in that context (with its device current) and cached under the context's
// unique id (cuCtxGetId): a caller on its own context (cuCtxCreate) or on a primary context created
// anew after cudaDeviceReset gets that context's own address, never one of another context.
#include <cuda.h>

#include <map>
#include <mutex>

#include "lbm_internal.h"
#include "reduce.cuh"

namespace lbm {
lbm_status set_thread_error(lbm_status s, const std::string &msg);
}

namespace {

constexpr int kRowsPerBlock = 4;
constexpr int kMaxRows = LBM_NOALLOC_MAX_ROWS;
constexpr int kMaxBlocks = kMaxRows / kRowsPerBlock;

// One (mass, momentum x, momentum y) partial per block of kRowsPerBlock rows.  Every block writes its
// own triple before the finaliser reads it, so nothing carries over from the previous call.
static __device__ __align__(256) double g_partials[kMaxBlocks * 3];

using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

std::mutex g_mu;
std::map<unsigned long long, double *> g_partials_addr;  // context id -> device address of g_partials
CtxGetIdFn g_ctx_get_id = nullptr;
bool g_ctx_get_id_looked_up = false;

// Unique id of the current context (0 when the driver entry point is unavailable or no context is
// current).  The driver function is reached through the runtime, so the library needs no link
// against libcuda.  Called with g_mu held.
unsigned long long current_context_id() {
    if (!g_ctx_get_id_looked_up) {
        g_ctx_get_id_looked_up = true;
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(fn);
    }
    unsigned long long id = 0;
    if (!g_ctx_get_id || g_ctx_get_id(nullptr, &id) != CUDA_SUCCESS) return 0;
    return id;
}

lbm_status symbol_address(double **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_partials);
    if (e != cudaSuccess || !p)
        return lbm::set_thread_error(LBM_ERR_CUDA, std::string("cudaGetSymbolAddress of the static partials: ") +
                                                       cudaGetErrorString(e));
    *out = static_cast<double *>(p);
    return LBM_OK;
}

// Device address of g_partials in the current context (looked up once per context).
lbm_status partials_in_current_context(double **out) {
    int dev = 0;
    const cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return lbm::set_thread_error(LBM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    std::lock_guard<std::mutex> lk(g_mu);
    unsigned long long id = current_context_id();
    if (id == 0) {
        // no context current yet: the symbol lookup makes the device's primary context current
        lbm_status st = symbol_address(out);
        if (st != LBM_OK) return st;
        id = current_context_id();
        if (id == 0) return LBM_OK;  // no context ids from this driver: the address just looked up
        g_partials_addr[id] = *out;
        return LBM_OK;
    }
    auto it = g_partials_addr.find(id);
    if (it != g_partials_addr.end()) {
        *out = it->second;
        return LBM_OK;
    }
    lbm_status st = symbol_address(out);
    if (st == LBM_OK) g_partials_addr[id] = *out;
    return st;
}

// FP64 sums of the unshifted populations over fluid cells, kRowsPerBlock rows per block
template <class T>
__global__ void __launch_bounds__(256) rows_kernel(const T *__restrict__ f, const uint8_t *__restrict__ flags, int nx,
                                                   int ny, int64_t row_pitch, double *__restrict__ partials) {
    double acc[3] = {0.0, 0.0, 0.0};
    const int64_t plane = row_pitch * ny;
    for (int r = 0; r < kRowsPerBlock; ++r) {
        const int y = blockIdx.x * kRowsPerBlock + r;
        if (y >= ny) break;
        for (int x = threadIdx.x; x < nx; x += blockDim.x) {
            if (flags[(int64_t)y * nx + x] != LBM_FLUID) continue;
            const int64_t c = (int64_t)y * row_pitch + x;
            double g[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) g[q] = (double)f[q * plane + c];
            double s = 0.0;
#pragma unroll
            for (int q = 0; q < 9; ++q) s += g[q];
            acc[0] += s;
            acc[1] += g[1] - g[3] + g[5] - g[6] - g[7] + g[8];
            acc[2] += g[2] - g[4] + g[5] + g[6] - g[7] - g[8];
        }
    }
    lbm::block_sum<3>(acc, partials + 3 * blockIdx.x);
}

}  // namespace

extern "C" LBM_API lbm_status lbm_d2q9_conservation_noalloc(const void *dev_populations, int32_t dtype,
                                                            const uint8_t *dev_flags, int32_t nx, int32_t ny,
                                                            int64_t row_pitch, double *dev_out, void *stream) {
    if (!dev_populations || !dev_flags || !dev_out)
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_d2q9_conservation_noalloc: null pointer");
    if (dtype != LBM_F32 && dtype != LBM_F64)
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_d2q9_conservation_noalloc: dtype must be LBM_F32 or LBM_F64");
    if (nx < 1 || ny < 1 || row_pitch < nx)
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_d2q9_conservation_noalloc: need nx >= 1, ny >= 1, row_pitch >= nx");
    if (ny > kMaxRows)
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_d2q9_conservation_noalloc: ny = " + std::to_string(ny) +
                                                          " rows exceeds the maximum of " + std::to_string(kMaxRows) +
                                                          " rows that its fixed scratch array holds");
    if (row_pitch > (((int64_t)1 << 40) / 9) / ny)  // 9 * row_pitch * ny > 2^40, without overflowing
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_d2q9_conservation_noalloc: population buffer too large");
    double *partials = nullptr;
    lbm_status st = partials_in_current_context(&partials);
    if (st != LBM_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nblocks = (ny + kRowsPerBlock - 1) / kRowsPerBlock;
    if (dtype == LBM_F32)
        rows_kernel<float><<<nblocks, 256, 0, s>>>(static_cast<const float *>(dev_populations), dev_flags, nx, ny,
                                                  row_pitch, partials);
    else
        rows_kernel<double><<<nblocks, 256, 0, s>>>(static_cast<const double *>(dev_populations), dev_flags, nx, ny,
                                                   row_pitch, partials);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = lbm::finalize_sums(s, partials, nblocks, 3, dev_out);
    if (e != cudaSuccess)
        return lbm::set_thread_error(LBM_ERR_CUDA, std::string("lbm_d2q9_conservation_noalloc: ") + cudaGetErrorString(e));
    return LBM_OK;
}
