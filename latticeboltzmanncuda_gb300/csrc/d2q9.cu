// D2Q9 kernels: fused pull step (streaming + half-way bounce-back + moving walls + periodic wrap +
// BGK collision + Guo forcing in one pass: one read and one write of the nine populations per
// cell update) in scalar, vectorised (d2q9_vec.cuh), bulk-copy (d2q9_bulk.cuh) and two-steps-per-
// launch (d2q9_tile2.cuh) forms chosen by an autotuner, link-word construction, equilibrium
// initialisation, moments, FP64 conservation sums and host-layout conversion.  The vectorised step
// is launched as the programmatic dependent of the launch before it (pdl.cuh), so back-to-back
// steps overlap one step's last wave with the next step's first blocks.
//
// Storage: structure of arrays, plane q holds population q of all cells, rows padded to `pitch`
// elements (a multiple of 32) so each row starts 128-byte aligned in FP32.  Populations are
// stored in the w-normalised shifted space h_q = s (f_q - w_q) / w_q (d2q9_core.cuh) in FP32 / FP16 /
// BF16 (arithmetic in FP32) or FP64 (the GPU oracle).  Two buffers (A/B): step n reads f[cur] and
// writes f[cur ^ 1].
//
// Population order: 0:(0,0) 1:(1,0) 2:(0,1) 3:(-1,0) 4:(0,-1) 5:(1,1) 6:(-1,1) 7:(-1,-1) 8:(1,-1).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>

#include "lbm_internal.h"
#include "d2q9_core.cuh"
#include "d2q9_bulk.cuh"
#include "d2q9_tile2.cuh"
#include "d2q9_vec.cuh"
#include "pdl.cuh"
#include "reduce.cuh"

namespace lbm {

D2Q9Params d2q9_params(const lbm_desc &d) {
    D2Q9Params p;
    p.omega_d = 1.0 / (double)d.tau;
    p.fx_d = d.body_force[0];
    p.fy_d = d.body_force[1];
    p.uwx_d = d.wall_velocity[0];
    p.uwy_d = d.wall_velocity[1];
    p.omega = (float)p.omega_d;
    p.fx = d.body_force[0];
    p.fy = d.body_force[1];
    p.uwx = d.wall_velocity[0];
    p.uwy = d.wall_velocity[1];
    return p;
}

namespace {

// ------------------------------------------------------------------------------------------------
// link words: one pass over the flag bytes
// ------------------------------------------------------------------------------------------------
// The step kernels never write a solid cell, so both population buffers must hold the same values
// there: a solid cell's populations are copied from the current buffer into the other one.
template <class W>
__device__ __forceinline__ void copy_cell(const void *cur, void *other, int64_t c, int64_t plane) {
    const W *a = static_cast<const W *>(cur);
    W *b = static_cast<W *>(other);
#pragma unroll
    for (int q = 0; q < 9; ++q) b[q * plane + c] = a[q * plane + c];
}

__global__ void build_links_kernel(const uint8_t *__restrict__ flags, uint16_t *__restrict__ links,
                                   int nx, int ny, int64_t pitch, int periodic, const void *cur, void *other,
                                   int elem) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= nx) return;
    int64_t c = (int64_t)y * pitch + x;
    if (flags[(int64_t)y * nx + x] != 0) {
        links[c] = LINK_SOLID;
        const int64_t plane = pitch * ny;
        if (elem == 2) copy_cell<uint16_t>(cur, other, c, plane);
        else if (elem == 4) copy_cell<uint32_t>(cur, other, c, plane);
        else copy_cell<uint64_t>(cur, other, c, plane);
        return;
    }
    uint16_t L = 0;
#pragma unroll
    for (int j = 1; j < 9; ++j) {
        int sx = x - d2q9::cx(j), sy = y - d2q9::cy(j);
        bool outside = false;
        if (sx < 0 || sx >= nx) {
            if (periodic & 1) sx = (sx + nx) % nx; else outside = true;
        }
        if (sy < 0 || sy >= ny) {
            if (periodic & 2) sy = (sy + ny) % ny; else outside = true;
        }
        if (outside) {
            L |= (uint16_t)(1u << (j - 1));
        } else {
            uint8_t fl = flags[(int64_t)sy * nx + sx];
            if (fl != 0) L |= (uint16_t)(1u << (j - 1));
            if (fl == LBM_MOVING_WALL) L |= (uint16_t)(1u << (j + 7));
        }
    }
    links[c] = L;
}

__global__ void count_fluid_kernel(const uint8_t *__restrict__ flags, int64_t n, unsigned long long *out) {
    unsigned long long local = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        local += flags[i] == 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(out, local);
}

// ------------------------------------------------------------------------------------------------
// fused step.  Rows are visited in increasing order on even sweeps and decreasing order on odd
// ones (`reverse`): a step then starts on the rows the previous step wrote last, which are still in
// L2, instead of on the rows it wrote first.
// ------------------------------------------------------------------------------------------------
template <class S, bool FORCE, class I>
__global__ void __launch_bounds__(256) step_kernel(const S *__restrict__ src, S *__restrict__ dst,
                                                   const uint16_t *__restrict__ links, int nx, int ny, I pitch,
                                                   I plane, int periodic, D2Q9Params prm, int reverse) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= nx || row >= ny) return;
    const int y = reverse ? ny - 1 - row : row;
    d2q9::scalar_cell<S, I>(src, dst, links, x, y, nx, ny, pitch, plane, periodic, prm, FORCE);
}

// Minimum resident blocks of 256 threads per SM asked of the register allocator, per vector width:
// 8-wide 16-bit vectors need their ~128 registers; narrower vectors trade a few spilled registers
// for more resident warps, which measured faster (the step is latency-bound at low occupancy).
__host__ __device__ constexpr int vec_min_blocks(int v) { return v == 8 ? 2 : 4; }

template <class S, int V, bool FORCE, int POL>
__global__ void __launch_bounds__(256, vec_min_blocks(V)) step_vec_kernel(const S *__restrict__ src, S *__restrict__ dst,
                                                       const uint16_t *__restrict__ links, int nx, int ny,
                                                       int pitch, int plane, int periodic, D2Q9Params prm,
                                                       int reverse) {
    // launched as the programmatic dependent of the step before: nothing is read before that step
    // has completed, and the next step's blocks may be scheduled as this one's last blocks finish
    wait_prerequisite_grids();
    allow_dependent_launch();
    const int row = blockIdx.y * blockDim.y + threadIdx.y;
    if (row >= ny) return;  // uniform per warp: warps never straddle rows
    const int y = reverse ? ny - 1 - row : row;
    const int x0 = (blockIdx.x * blockDim.x + threadIdx.x) * V;
    d2q9::step_vec<S, V, FORCE, int, POL>(src, dst, links, x0, y, nx, ny, pitch, plane, periodic, prm);
}

// 16-bit storage: the bulk-copy pipeline (d2q9_bulk.cuh), persistent blocks over (strip, row) tasks
template <class S, int V, bool FORCE, int K, int MINB>
__global__ void __launch_bounds__(d2q9::bulk::threads<V>(), MINB)
    bulk_kernel(const S *__restrict__ src, S *__restrict__ dst, const uint16_t *__restrict__ links, int nx, int ny,
                int pitch, int plane, int periodic, D2Q9Params prm, int reverse, unsigned *status,
                unsigned long long wait_ns, int skip_task) {
    extern __shared__ __align__(128) unsigned char smem[];
    d2q9::bulk::pipeline<S, V, FORCE, K>(smem, src, dst, links, nx, ny, pitch, plane, periodic, prm, reverse, status,
                                         wait_ns, skip_task);
}

// Resident blocks of a kernel per SM times the SMs of `device` (cached per kernel and device).
int resident_blocks(const void *kernel, int threads, size_t smem, int device) {
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, int> cache;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find({kernel, device});
    if (it != cache.end()) return it->second;
    int per_sm = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return 0;
    return cache[{kernel, device}] = std::max(1, per_sm) * sms;
}

// launch the bulk-copy pipeline (V cells per consumer thread) with a ring of K slots, registers
// bounded for MINB blocks per SM (the dynamic shared memory is opted in once per kernel and
// device); one persistent block per resident slot, at most one per task
template <class S, int V, bool FORCE, int K, int MINB>
cudaError_t launch_bulk(lbm_ctx *ctx, const S *src, S *dst, int reverse) {
    namespace B = d2q9::bulk;
    constexpr size_t bytes = B::smem_bytes<K>();
    constexpr int threads = B::threads<V>();
    auto kern = bulk_kernel<S, V, FORCE, K, MINB>;
    static std::mutex mu;
    static unsigned long long opted = 0;  // devices on which the attribute is set
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!(opted >> (ctx->device & 63) & 1ull)) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
            if (e != cudaSuccess) return e;
            opted |= 1ull << (ctx->device & 63);
        }
    }
    const lbm_desc &d = ctx->desc;
    const int pitch = (int)ctx->pitch, plane = (int)ctx->plane;
    const int ntasks = ((pitch + B::W - 1) / B::W) * d.ny;
    const int resident = resident_blocks(reinterpret_cast<const void *>(kern), threads, bytes, ctx->device);
    if (resident <= 0) return cudaErrorInvalidConfiguration;
    const int grid = std::min(ntasks, resident);
    ctx->pipe_used = true;
    kern<<<grid, threads, bytes, ctx->stream>>>(src, dst, ctx->links_d, d.nx, d.ny, pitch, plane, d.periodic,
                                                d2q9_params(d), reverse, ctx->pipe_status_d, ctx->pipe_wait_ns,
                                                ctx->pipe_skip_task);
    return cudaGetLastError();
}

// pipeline variants (4 cells per consumer thread; 2 measured slower on the FP16 channel, 78-88k
// against 96-104k MLUPS): pol selects the ring depth and the register bound (0: 4 slots, 5 blocks
// per SM; 1: 4 slots, 4 blocks; 2: 6 slots, 3 blocks)
template <class S, bool FORCE>
cudaError_t launch_bulk_variant(lbm_ctx *ctx, int pol, const S *src, S *dst, int reverse) {
    if (pol == 0) return launch_bulk<S, 4, FORCE, 4, 5>(ctx, src, dst, reverse);
    if (pol == 1) return launch_bulk<S, 4, FORCE, 4, 4>(ctx, src, dst, reverse);
    return launch_bulk<S, 4, FORCE, 6, 3>(ctx, src, dst, reverse);
}

template <class S>
__global__ void moments_kernel(const S *__restrict__ src, const uint16_t *__restrict__ links, int nx,
                               int ny, int64_t pitch, int64_t plane, int periodic, D2Q9Params prm,
                               float *__restrict__ rho_o, float *__restrict__ ux_o, float *__restrict__ uy_o) {
    using R = typename d2q9::Store<S>::R;
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= nx) return;
    int64_t c = (int64_t)y * pitch + x;
    int64_t o = (int64_t)y * nx + x;
    uint16_t L = links[c];
    R rho = 1, ux = 0, uy = 0;
    if (L != LINK_SOLID) {
        R h[9];
        d2q9::gather<S, R>(src, L, x, y, nx, ny, pitch, plane, periodic, d2q9::wall_u<R>(prm), h);
        R drho, mx, my;
        d2q9::moments<S, R>(h, drho, mx, my);
        rho = (R)1 + drho;
        const auto F = d2q9::force<R>(prm);
        ux = (mx + (R)0.5 * F.x) / rho;
        uy = (my + (R)0.5 * F.y) / rho;
    }
    if (rho_o) rho_o[o] = (float)rho;
    if (ux_o) ux_o[o] = (float)ux;
    if (uy_o) uy_o[o] = (float)uy;
}

template <class S>
__global__ void equilibrium_kernel(S *__restrict__ a, S *__restrict__ b, int nx, int ny, int64_t pitch,
                                   int64_t plane, const float *__restrict__ rho, const float *__restrict__ ux,
                                   const float *__restrict__ uy) {
    using R = typename d2q9::Store<S>::R;
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= nx) return;
    int64_t o = (int64_t)y * nx + x;
    int64_t c = (int64_t)y * pitch + x;
    R r = rho ? (R)rho[o] : (R)1, u = ux ? (R)ux[o] : (R)0, v = uy ? (R)uy[o] : (R)0;
    R h[9];
    d2q9::equilibrium_h<S, R>(r - (R)1, r, u, v, h);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        d2q9::sth<S>(a + q * plane + c, h[q]);
        d2q9::sth<S>(b + q * plane + c, h[q]);
    }
}

// FP64 sums of mass and momentum of the stored populations over fluid cells; one partial per block
template <class S>
__global__ void conservation_kernel(const S *__restrict__ src, const uint16_t *__restrict__ links, int nx,
                                    int ny, int64_t pitch, int64_t plane, double *__restrict__ partials) {
    double m = 0, px = 0, py = 0;
    int64_t n = (int64_t)nx * ny;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t y = i / nx, x = i - y * nx;
        int64_t c = y * pitch + x;
        if (links[c] == LINK_SOLID) continue;
        double g[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) g[q] = (double)d2q9::ldq<S>(src + q * plane + c, q);
        double s = 0;
#pragma unroll
        for (int q = 0; q < 9; ++q) s += g[q];
        m += 1.0 + s;
        px += g[1] - g[3] + g[5] - g[6] - g[7] + g[8];
        py += g[2] - g[4] + g[5] + g[6] - g[7] - g[8];
    }
    double acc[3] = {m, px, py};
    block_sum<3>(acc, partials + 3 * blockIdx.x);
}

// host layout <-> device storage.  aos: struct LatticePoint records (144 bytes, floats from
// byte 12, record index y + ny*x); else unshifted SoA [9][ny][nx] in float or double.
__device__ __forceinline__ int aos_slot(int q) {
    // reference slots of the in-plane D3Q27 directions (SimCalcFuncs.cu:12)
    constexpr int s[9] = {0, 6, 5, 1, 2, 18, 10, 7, 15};
    return s[q];
}

template <class S, class H>
__global__ void load_kernel(S *__restrict__ a, S *__restrict__ b, const H *__restrict__ host, int nx, int ny,
                            int64_t pitch, int64_t plane, int aos) {
    using R = typename d2q9::Store<S>::R;
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= nx) return;
    int64_t c = (int64_t)y * pitch + x;
    int64_t n = (int64_t)nx * ny;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        R v;
        if (aos) {
            const char *rec = reinterpret_cast<const char *>(host) + ((int64_t)y + (int64_t)ny * x) * 144;
            v = (R)(reinterpret_cast<const float *>(rec + 12)[aos_slot(q)]);
        } else {
            v = (R)host[q * n + (int64_t)y * nx + x];
        }
        R g = v - d2q9::w<R>(q);
        d2q9::stq<S>(a + q * plane + c, q, g);
        d2q9::stq<S>(b + q * plane + c, q, g);
    }
}

template <class S, class H>
__global__ void store_kernel(const S *__restrict__ src, H *__restrict__ host, int nx, int ny, int64_t pitch,
                             int64_t plane, int aos, const uint8_t *__restrict__ flags) {
    using R = typename d2q9::Store<S>::R;
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= nx) return;
    int64_t c = (int64_t)y * pitch + x;
    int64_t n = (int64_t)nx * ny;
    if (aos) {
        char *rec = reinterpret_cast<char *>(host) + ((int64_t)y + (int64_t)ny * x) * 144;
        int *xyz = reinterpret_cast<int *>(rec);
        xyz[0] = x;
        xyz[1] = y;
        xyz[2] = 0;
        float *f = reinterpret_cast<float *>(rec + 12);
        for (int k = 0; k < 27; ++k) f[k] = 0.0f;
#pragma unroll
        for (int q = 0; q < 9; ++q) f[aos_slot(q)] = (float)(d2q9::ldq<S>(src + q * plane + c, q) + d2q9::w<R>(q));
        uint8_t fl = flags ? flags[(int64_t)y * nx + x] : 0;
        rec[120] = 0;        // isReflected
        rec[121] = fl != 0;  // isInternal: solid cell
        *reinterpret_cast<unsigned long long *>(rec + 128) = 0ull;
        *reinterpret_cast<unsigned long long *>(rec + 136) = 0ull;
    } else {
#pragma unroll
        for (int q = 0; q < 9; ++q)
            host[q * n + (int64_t)y * nx + x] = (H)d2q9::ldq<S>(src + q * plane + c, q) + d2q9::w<H>(q);
    }
}

// ------------------------------------------------------------------------------------------------
// launch shapes and the autotuner
// ------------------------------------------------------------------------------------------------
struct Shape {
    int v, tx, ty, pol;  // cells per thread, block shape, L2 policy of the vector path (0, 1, 2)
};

// v == TILE2: two steps per launch on shared-memory tiles of tx x ty cells (d2q9_tile2.cuh)
constexpr int TILE2 = -2;

template <class S, int TX, int TY, bool FORCE>
__global__ void __launch_bounds__(d2q9::tile2::THREADS) tile2_kernel(const S *__restrict__ src, S *__restrict__ dst,
                                                                    const uint16_t *__restrict__ links, int nx,
                                                                    int ny, int pitch, int plane, int periodic,
                                                                    D2Q9Params prm) {
    extern __shared__ __align__(16) unsigned char smem[];
    d2q9::tile2::two_steps<S, TX, TY, FORCE>(src, dst, links, nx, ny, pitch, plane, periodic, prm, smem);
}

template <class S, int TX, int TY, bool FORCE>
cudaError_t launch_tile2_t(lbm_ctx *ctx, const S *src, S *dst, const D2Q9Params &prm) {
    constexpr size_t bytes = d2q9::tile2::Layout<S, TX, TY>::bytes;
    static bool attr_set = false;  // per instantiation (the attribute is per function)
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(tile2_kernel<S, TX, TY, FORCE>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const lbm_desc &d = ctx->desc;
    const dim3 grid((unsigned)((d.nx + TX - 1) / TX), (unsigned)((d.ny + TY - 1) / TY));
    tile2_kernel<S, TX, TY, FORCE><<<grid, d2q9::tile2::THREADS, bytes, ctx->stream>>>(
        src, dst, ctx->links_d, d.nx, d.ny, (int)ctx->pitch, (int)ctx->plane, d.periodic, prm);
    return cudaGetLastError();
}

// the tile shapes of the two-step kernel
inline bool tile2_shape(int tx, int ty) { return (tx == 64 && (ty == 8 || ty == 16)) || (tx == 128 && ty == 8); }

// v == TILE2P: the persistent two-step kernel (the next tile's copies in flight while a tile is
// computed), tiles of 64 x 4 or 64 x 8 cells
constexpr int TILE2P = -3;
inline bool tile2p_shape(int tx, int ty) { return tx == 64 && (ty == 4 || ty == 8); }

// 256 threads a block (512 measured slower: FP32 81.8k against 83.3k MLUPS on 64 x 8 tiles)
constexpr int TILE2P_THREADS = 256;

template <class S, int TX, int TY, bool FORCE>
__global__ void __launch_bounds__(TILE2P_THREADS) tile2p_kernel(const S *__restrict__ src, S *__restrict__ dst,
                                                                     const uint16_t *__restrict__ links, int nx,
                                                                     int ny, int pitch, int plane, int periodic,
                                                                     D2Q9Params prm, int tiles_x, int ntiles) {
    extern __shared__ __align__(16) unsigned char smem[];
    d2q9::tile2::two_steps_persistent<S, TX, TY, FORCE, TILE2P_THREADS>(src, dst, links, nx, ny, pitch, plane,
                                                                        periodic, prm, smem, tiles_x, ntiles);
}

template <class S, int TX, int TY, bool FORCE>
cudaError_t launch_tile2p_t(lbm_ctx *ctx, const S *src, S *dst, const D2Q9Params &prm) {
    constexpr size_t bytes = d2q9::tile2::LayoutP<S, TX, TY>::bytes;
    static int per_sm = 0;  // per instantiation: resident blocks per SM, from the occupancy calculator
    if (per_sm == 0) {
        cudaError_t e = cudaFuncSetAttribute(tile2p_kernel<S, TX, TY, FORCE>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tile2p_kernel<S, TX, TY, FORCE>,
                                                              TILE2P_THREADS, bytes);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorInvalidConfiguration;
    }
    int sms = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e != cudaSuccess) return e;
    const lbm_desc &d = ctx->desc;
    const int tiles_x = (d.nx + TX - 1) / TX, ntiles = tiles_x * ((d.ny + TY - 1) / TY);
    const int grid = std::min(ntiles, per_sm * sms);
    tile2p_kernel<S, TX, TY, FORCE><<<grid, TILE2P_THREADS, bytes, ctx->stream>>>(
        src, dst, ctx->links_d, d.nx, d.ny, (int)ctx->pitch, (int)ctx->plane, d.periodic, prm, tiles_x, ntiles);
    return cudaGetLastError();
}

template <class S>
cudaError_t launch_tile2p(lbm_ctx *ctx, int tx, int ty, const S *src, S *dst) {
    if constexpr (sizeof(S) > 4) {
        return cudaErrorInvalidValue;
    } else {
        const D2Q9Params prm = d2q9_params(ctx->desc);
        const bool f = prm.fx != 0.0f || prm.fy != 0.0f;
        if (tx == 64 && ty == 4) return f ? launch_tile2p_t<S, 64, 4, true>(ctx, src, dst, prm) : launch_tile2p_t<S, 64, 4, false>(ctx, src, dst, prm);
        if (tx == 64 && ty == 8) return f ? launch_tile2p_t<S, 64, 8, true>(ctx, src, dst, prm) : launch_tile2p_t<S, 64, 8, false>(ctx, src, dst, prm);
        return cudaErrorInvalidValue;
    }
}

template <class S>
cudaError_t launch_tile2(lbm_ctx *ctx, int tx, int ty, const S *src, S *dst) {
    if constexpr (sizeof(S) > 4) {
        return cudaErrorInvalidValue;
    } else {
        const D2Q9Params prm = d2q9_params(ctx->desc);
        const bool f = prm.fx != 0.0f || prm.fy != 0.0f;
        if (tx == 64 && ty == 8) return f ? launch_tile2_t<S, 64, 8, true>(ctx, src, dst, prm) : launch_tile2_t<S, 64, 8, false>(ctx, src, dst, prm);
        if (tx == 64 && ty == 16) return f ? launch_tile2_t<S, 64, 16, true>(ctx, src, dst, prm) : launch_tile2_t<S, 64, 16, false>(ctx, src, dst, prm);
        if (tx == 128 && ty == 8) return f ? launch_tile2_t<S, 128, 8, true>(ctx, src, dst, prm) : launch_tile2_t<S, 128, 8, false>(ctx, src, dst, prm);
        return cudaErrorInvalidValue;
    }
}

template <class S>
constexpr bool vec_ok(int v) {
    return (sizeof(S) == 4 && (v == 2 || v == 4)) || (sizeof(S) == 2 && (v == 2 || v == 4 || v == 8)) ||
           (sizeof(S) == 8 && v == 2);
}

bool small_index(const lbm_ctx *ctx) { return ctx->plane * 9 < (int64_t)INT32_MAX; }

template <class S>
cudaError_t launch_one(lbm_ctx *ctx, const Shape &sh, const S *src, S *dst, int reverse) {
    const lbm_desc &d = ctx->desc;
    const D2Q9Params prm = d2q9_params(d);
    const bool force = prm.fx != 0.0f || prm.fy != 0.0f;
    dim3 block(sh.tx, sh.ty);
    const int per_row = sh.v == 1 ? d.nx : (int)(ctx->pitch / sh.v);
    dim3 grid((unsigned)((per_row + sh.tx - 1) / sh.tx), (unsigned)((d.ny + sh.ty - 1) / sh.ty));
    cudaStream_t st = ctx->stream;
    if (sh.v == 1) {
        if (small_index(ctx)) {
            const int pitch = (int)ctx->pitch, plane = (int)ctx->plane;
            if (force) step_kernel<S, true, int><<<grid, block, 0, st>>>(src, dst, ctx->links_d, d.nx, d.ny, pitch, plane, d.periodic, prm, reverse);
            else step_kernel<S, false, int><<<grid, block, 0, st>>>(src, dst, ctx->links_d, d.nx, d.ny, pitch, plane, d.periodic, prm, reverse);
        } else {
            if (force) step_kernel<S, true, int64_t><<<grid, block, 0, st>>>(src, dst, ctx->links_d, d.nx, d.ny, ctx->pitch, ctx->plane, d.periodic, prm, reverse);
            else step_kernel<S, false, int64_t><<<grid, block, 0, st>>>(src, dst, ctx->links_d, d.nx, d.ny, ctx->pitch, ctx->plane, d.periodic, prm, reverse);
        }
        return cudaGetLastError();
    }
    if (sh.v == TILE2) return launch_tile2<S>(ctx, sh.tx, sh.ty, src, dst);    // two steps
    if (sh.v == TILE2P) return launch_tile2p<S>(ctx, sh.tx, sh.ty, src, dst);  // two steps, persistent
    const int pitch = (int)ctx->pitch, plane = (int)ctx->plane;
    if (sh.v == 0) {  // bulk-copy pipeline
        if constexpr (sizeof(S) == 2)
            return force ? launch_bulk_variant<S, true>(ctx, sh.pol, src, dst, reverse)
                         : launch_bulk_variant<S, false>(ctx, sh.pol, src, dst, reverse);
        return cudaErrorInvalidValue;
    }
    // the vector kernels: programmatic dependents of the launch before (back-to-back steps overlap
    // one step's last blocks with the next one's launch)
#define LBM_VEC_LAUNCH(VV, PP)                                                                                  \
    e = force ? launch_maybe_dependent(true, step_vec_kernel<S, VV, true, PP>, grid, block, 0, st, src, dst,    \
                                       links, d.nx, d.ny, pitch, plane, d.periodic, prm, reverse)               \
              : launch_maybe_dependent(true, step_vec_kernel<S, VV, false, PP>, grid, block, 0, st, src, dst,   \
                                       links, d.nx, d.ny, pitch, plane, d.periodic, prm, reverse);
#define LBM_VEC_CASE(VV)                                                                                        \
    if constexpr (vec_ok<S>(VV)) {                                                                              \
        if (sh.v == VV) {                                                                                       \
            cudaError_t e;                                                                                      \
            if (sh.pol == 1) { LBM_VEC_LAUNCH(VV, 1) }                                                          \
            else if (sh.pol == 2) { LBM_VEC_LAUNCH(VV, 2) }                                                     \
            else { LBM_VEC_LAUNCH(VV, 0) }                                                                      \
            return e != cudaSuccess ? e : cudaGetLastError();                                                   \
        }                                                                                                       \
    }
    const uint16_t *links = ctx->links_d;
    LBM_VEC_CASE(2)
    LBM_VEC_CASE(4)
    LBM_VEC_CASE(8)
#undef LBM_VEC_CASE
#undef LBM_VEC_LAUNCH
    return cudaErrorInvalidValue;
}

template <class S>
std::vector<Shape> candidates(const lbm_ctx *ctx) {
    std::vector<Shape> c = {{1, 256, 1, 0}, {1, 128, 2, 0}};
    if (!small_index(ctx)) return c;
    if (sizeof(S) == 2)  // the bulk-copy pipeline
        for (int pol : {0, 1, 2}) c.push_back({0, d2q9::bulk::threads<4>(), 1, pol});
    if (sizeof(S) <= 4) {  // two steps per launch on shared-memory tiles
        for (const auto &t : {std::pair<int, int>{64, 8}, {64, 16}, {128, 8}}) c.push_back({TILE2, t.first, t.second, 0});
        for (int ty : {4, 8}) c.push_back({TILE2P, 64, ty, 0});
    }
    for (int v : {2, 4, 8}) {
        if (!vec_ok<S>(v) || ctx->pitch % v) continue;
        const int per_row = (int)(ctx->pitch / v);
        for (int tx : {32, 64, 128, 256}) {
            if (tx > 32 && tx / 2 >= per_row) continue;  // a block wider than two rows' worth is idle
            const int ty = std::max(1, std::min(256 / tx, 4));
            for (int pol = 0; pol < 3; ++pol) {
                c.push_back({v, tx, 1, pol});
                if (ty > 1 && tx * ty <= 256) c.push_back({v, tx, ty, pol});
            }
        }
    }
    return c;
}

std::mutex g_tune_mu;
std::map<std::string, Shape> g_tune_cache;
bool g_tune_file_loaded = false;

std::string tune_key(const lbm_ctx *ctx) {
    const lbm_desc &d = ctx->desc;
    const bool force = d.body_force[0] != 0.0f || d.body_force[1] != 0.0f;
    char buf[128];
    std::snprintf(buf, sizeof(buf), "d2q9/%d/%dx%d/p%d/f%d", d.dtype, d.nx, d.ny, d.periodic, force ? 1 : 0);
    return buf;
}

std::string tune_path() {
    const char *e = std::getenv("LBM_TUNE_CACHE");
    if (e) return e;  // empty: no file cache
    const char *xdg = std::getenv("XDG_CACHE_HOME");
    const char *home = std::getenv("HOME");
    if (xdg && *xdg) return std::string(xdg) + "/lbm_gb300_tune.json";
    if (home && *home) return std::string(home) + "/.cache/lbm_gb300_tune.json";
    return "";
}

// flat JSON object {"key": [v, tx, ty], ...}
void load_tune_file() {
    if (g_tune_file_loaded) return;
    g_tune_file_loaded = true;
    const std::string path = tune_path();
    if (path.empty()) return;
    FILE *fp = std::fopen(path.c_str(), "r");
    if (!fp) return;
    std::string txt;
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), fp)) > 0) txt.append(buf, n);
    std::fclose(fp);
    size_t pos = 0;
    while ((pos = txt.find('"', pos)) != std::string::npos) {
        const size_t end = txt.find('"', pos + 1);
        if (end == std::string::npos) break;
        const std::string key = txt.substr(pos + 1, end - pos - 1);
        Shape sh{0, 0, 0, 0};
        if (std::sscanf(txt.c_str() + end + 1, " : [ %d , %d , %d , %d ]", &sh.v, &sh.tx, &sh.ty, &sh.pol) == 4 && sh.v >= 0 &&
            sh.tx > 0 && sh.ty > 0)
            g_tune_cache[key] = sh;
        pos = end + 1;
    }
}

void save_tune_file() {
    const std::string path = tune_path();
    if (path.empty()) return;
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos && slash > 0) mkdir(path.substr(0, slash).c_str(), 0755);  // may exist
    const std::string tmp = path + ".tmp";
    FILE *fp = std::fopen(tmp.c_str(), "w");
    if (!fp) return;
    std::fprintf(fp, "{\n");
    size_t i = 0;
    for (const auto &kv : g_tune_cache)
        std::fprintf(fp, "  \"%s\": [%d, %d, %d, %d]%s\n", kv.first.c_str(), kv.second.v, kv.second.tx, kv.second.ty,
                     kv.second.pol, ++i < g_tune_cache.size() ? "," : "");
    std::fprintf(fp, "}\n");
    std::fclose(fp);
    std::rename(tmp.c_str(), path.c_str());
}

// Time every candidate shape on the context's own domain (f[cur] -> f[cur^1] repeatedly, without
// swapping, so the state is unchanged), then time the four fastest again with four times the
// launches, in forward and reverse order, and keep the fastest of those (shapes within a few per
// cent of each other are otherwise picked by timing noise).
template <class S>
cudaError_t tune(lbm_ctx *ctx) {
    const S *src = static_cast<const S *>(ctx->f[ctx->cur]);
    S *dst = static_cast<S *>(ctx->f[ctx->cur ^ 1]);
    cudaEvent_t e0, e1;
    cudaError_t err = cudaEventCreate(&e0);
    if (err != cudaSuccess) return err;
    err = cudaEventCreate(&e1);
    if (err != cudaSuccess) {
        cudaEventDestroy(e0);
        return err;
    }
    const int64_t cells = (int64_t)ctx->desc.nx * ctx->desc.ny;
    const int reps = cells > (1 << 22) ? 6 : (cells > (1 << 18) ? 12 : 30);
    // ms of `n` launches of shape sh after two warm-up launches; < 0 when the shape is not usable
    auto time_shape = [&](const Shape &sh, int n, float &ms) -> cudaError_t {
        ms = -1.0f;
        cudaError_t e = cudaSuccess;
        for (int w = 0; w < 2 && e == cudaSuccess; ++w) e = launch_one<S>(ctx, sh, src, dst, w & 1);
        if (e != cudaSuccess) return e;
        cudaEventRecord(e0, ctx->stream);
        for (int r = 0; r < n && e == cudaSuccess; ++r) e = launch_one<S>(ctx, sh, src, dst, r & 1);
        cudaEventRecord(e1, ctx->stream);
        if (e != cudaSuccess) return e;
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) return e;
        float t = 0.0f;
        cudaEventElapsedTime(&t, e0, e1);
        if (sh.v == 0 && d2q9_take_pipe_status(ctx) != 0) return cudaSuccess;  // a bounded wait gave up
        ms = (sh.v == TILE2 || sh.v == TILE2P) ? 0.5f * t : t;  // per time step: a two-step launch counts twice
        return cudaSuccess;
    };
    const std::vector<Shape> cands = candidates<S>(ctx);
    // bring the clocks up before anything is compared: about 20 ms of launches of the first shape
    if (!cands.empty()) {
        float ms = -1.0f;
        err = time_shape(cands[0], 8, ms);
        if (err == cudaSuccess && ms > 0.0f) {
            const int n = (int)std::min(2000.0f, 20.0f / (ms / 8.0f));
            if (n > 8) err = time_shape(cands[0], n, ms);
        }
    }
    std::vector<std::pair<float, Shape>> timed;
    for (size_t i = 0; i < cands.size() && err == cudaSuccess; ++i) {
        float ms;
        if ((err = time_shape(cands[i], reps, ms)) != cudaSuccess) break;
        if (ms >= 0.0f) timed.push_back({ms, cands[i]});
    }
    Shape pick = {1, 256, 1, 0};
    if (err == cudaSuccess && !timed.empty()) {
        std::stable_sort(timed.begin(), timed.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
        // the four fastest again, four interleaved passes in alternating order with eight times the
        // launches (shapes a few per cent apart were otherwise picked by timing noise)
        const size_t top = std::min<size_t>(4, timed.size());
        std::vector<float> total(top, 0.0f);
        for (int pass = 0; pass < 4 && err == cudaSuccess; ++pass)
            for (size_t k = 0; k < top && err == cudaSuccess; ++k) {
                const size_t c = (pass & 1) ? top - 1 - k : k;
                float ms;
                err = time_shape(timed[c].second, 8 * reps, ms);
                total[c] = (ms < 0.0f || total[c] < 0.0f) ? -1.0f : total[c] + ms;
            }
        float best = 1e30f;
        pick = timed[0].second;
        for (size_t k = 0; k < top; ++k)
            if (total[k] >= 0.0f && total[k] < best) {
                best = total[k];
                pick = timed[k].second;
            }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) return err;
    ctx->cells_per_thread = pick.v;
    ctx->block_threads = pick.tx;
    ctx->rows_per_block = pick.ty;
    ctx->l2_policy = pick.pol;
    ctx->tuned = true;
    return cudaSuccess;
}

template <class S>
cudaError_t launch_step(lbm_ctx *ctx, int nsteps) {
    if (!ctx->tuned) {
        cudaError_t e = d2q9_autotune(ctx, false);
        if (e != cudaSuccess) return e;
    }
    const Shape sh{ctx->cells_per_thread, ctx->block_threads, ctx->rows_per_block, ctx->l2_policy};
    if (sh.v == TILE2 || sh.v == TILE2P) {
        // two steps per launch; an odd last step by the one-step vector kernel (bit-identical)
        for (int s = 0; s + 1 < nsteps; s += 2) {
            cudaError_t e = launch_one<S>(ctx, sh, static_cast<const S *>(ctx->f[ctx->cur]),
                                          static_cast<S *>(ctx->f[ctx->cur ^ 1]), 0);
            if (e != cudaSuccess) return e;
            ctx->cur ^= 1;
        }
        if (nsteps & 1) {
            const Shape one{2, 64, 1, 0};
            cudaError_t e = launch_one<S>(ctx, one, static_cast<const S *>(ctx->f[ctx->cur]),
                                          static_cast<S *>(ctx->f[ctx->cur ^ 1]), 0);
            if (e != cudaSuccess) return e;
            ctx->cur ^= 1;
        }
        return cudaSuccess;
    }
    for (int s = 0; s < nsteps; ++s) {
        const S *src = static_cast<const S *>(ctx->f[ctx->cur]);
        S *dst = static_cast<S *>(ctx->f[ctx->cur ^ 1]);
        const int reverse = ctx->alternate_sweeps ? (int)(ctx->sweep & 1) : 0;
        cudaError_t e = launch_one<S>(ctx, sh, src, dst, reverse);
        if (e != cudaSuccess) return e;
        ctx->sweep ^= 1;
        ctx->cur ^= 1;
    }
    return cudaSuccess;
}

template <class F>
cudaError_t dispatch(int dtype, F &&fn) {
    switch (dtype) {
        case LBM_F32: return fn(float{});
        case LBM_F16S: return fn(__half{});
        case LBM_BF16S: return fn(__nv_bfloat16{});
        case LBM_F64: return fn(double{});
    }
    return cudaErrorInvalidValue;
}

inline dim3 row_grid(const lbm_ctx *ctx, int threads) {
    return dim3((unsigned)((ctx->desc.nx + threads - 1) / threads), (unsigned)ctx->desc.ny);
}

}  // namespace

cudaError_t d2q9_build_links_async(lbm_ctx *ctx, unsigned long long *count_d) {
    const lbm_desc &d = ctx->desc;
    build_links_kernel<<<row_grid(ctx, 256), 256, 0, ctx->stream>>>(ctx->flags_d, ctx->links_d, d.nx, d.ny,
                                                                    ctx->pitch, d.periodic, ctx->f[ctx->cur],
                                                                    ctx->f[ctx->cur ^ 1], (int)ctx->elem);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemsetAsync(count_d, 0, sizeof(unsigned long long), ctx->stream);
    if (e != cudaSuccess) return e;
    count_fluid_kernel<<<256, 256, 0, ctx->stream>>>(ctx->flags_d, (int64_t)d.nx * d.ny, count_d);
    return cudaGetLastError();
}

cudaError_t d2q9_build_links(lbm_ctx *ctx) {
    const lbm_desc &d = ctx->desc;
    build_links_kernel<<<row_grid(ctx, 256), 256, 0, ctx->stream>>>(ctx->flags_d, ctx->links_d, d.nx, d.ny,
                                                                    ctx->pitch, d.periodic, ctx->f[ctx->cur],
                                                                    ctx->f[ctx->cur ^ 1], (int)ctx->elem);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(ctx->result_d);
    e = cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), ctx->stream);
    if (e != cudaSuccess) return e;
    count_fluid_kernel<<<256, 256, 0, ctx->stream>>>(ctx->flags_d, (int64_t)d.nx * d.ny, cnt);
    unsigned long long h = 0;
    e = cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(ctx->stream);
    ctx->fluid_cells = (int64_t)h;
    return e;
}

cudaError_t d2q9_init_equilibrium(lbm_ctx *ctx, const float *rho_d, const float *ux_d, const float *uy_d) {
    return dispatch(ctx->desc.dtype, [&](auto tag) {
        using S = decltype(tag);
        equilibrium_kernel<S><<<row_grid(ctx, 256), 256, 0, ctx->stream>>>(
            static_cast<S *>(ctx->f[0]), static_cast<S *>(ctx->f[1]), ctx->desc.nx, ctx->desc.ny, ctx->pitch,
            ctx->plane, rho_d, ux_d, uy_d);
        return cudaGetLastError();
    });
}

bool d2q9_shape_valid(const lbm_ctx *ctx, int v, int tx, int ty, int pol) {
    if (v == TILE2)  // two-step tiles: FP32 and 16-bit storage
        return ctx->desc.dtype != LBM_F64 && tile2_shape(tx, ty) && pol == 0 && small_index(ctx);
    if (v == TILE2P)  // persistent two-step tiles
        return ctx->desc.dtype != LBM_F64 && tile2p_shape(tx, ty) && pol == 0 && small_index(ctx);
    if (v == 0)  // bulk-copy pipeline: 16-bit storage, fixed block shape, three ring variants
        return (ctx->desc.dtype == LBM_F16S || ctx->desc.dtype == LBM_BF16S) &&
               tx == d2q9::bulk::threads<4>() && ty == 1 &&
               pol >= 0 && pol <= 2 && small_index(ctx);
    if (tx < 32 || tx % 32 || ty < 1 || tx * ty > 256 || pol < 0 || pol > 2) return false;
    if (v == 1) return pol == 0;
    if (!small_index(ctx) || ctx->pitch % v) return false;
    switch (ctx->desc.dtype) {
        case LBM_F32: return vec_ok<float>(v);
        case LBM_F16S: return vec_ok<__half>(v);
        case LBM_BF16S: return vec_ok<__nv_bfloat16>(v);
        case LBM_F64: return vec_ok<double>(v);
    }
    return false;
}

cudaError_t d2q9_autotune(lbm_ctx *ctx, bool force_retune) {
    const char *env = std::getenv("LBM_AUTOTUNE");
    const std::string key = tune_key(ctx);
    // LBM_D2Q9_LAUNCH="v,tx,ty" fixes the shape (reproducible profiling); ignored when not valid
    if (const char *fixed = std::getenv("LBM_D2Q9_LAUNCH")) {
        Shape sh{0, 0, 0, 0};
        if (std::sscanf(fixed, "%d,%d,%d,%d", &sh.v, &sh.tx, &sh.ty, &sh.pol) >= 3 &&
            d2q9_shape_valid(ctx, sh.v, sh.tx, sh.ty, sh.pol)) {
            ctx->cells_per_thread = sh.v;
            ctx->block_threads = sh.tx;
            ctx->rows_per_block = sh.ty;
            ctx->l2_policy = sh.pol;
            ctx->tuned = true;
            return cudaSuccess;
        }
    }
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        load_tune_file();
        auto it = g_tune_cache.find(key);
        if (!force_retune && it != g_tune_cache.end() &&
            d2q9_shape_valid(ctx, it->second.v, it->second.tx, it->second.ty, it->second.pol)) {
            ctx->cells_per_thread = it->second.v;
            ctx->block_threads = it->second.tx;
            ctx->rows_per_block = it->second.ty;
            ctx->l2_policy = it->second.pol;
            ctx->tuned = true;
            return cudaSuccess;
        }
    }
    if (env && env[0] == '0' && !force_retune) {
        // tuning switched off: the default shape
        const bool vec = d2q9_shape_valid(ctx, ctx->desc.dtype == LBM_F64 ? 2 : 4, 64, 1, 0);
        ctx->cells_per_thread = vec ? (ctx->desc.dtype == LBM_F64 ? 2 : 4) : 1;
        ctx->block_threads = vec ? 64 : 256;
        ctx->rows_per_block = 1;
        ctx->l2_policy = 0;
        ctx->tuned = true;
        return cudaSuccess;
    }
    cudaError_t e = dispatch(ctx->desc.dtype, [&](auto tag) { return tune<decltype(tag)>(ctx); });
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = Shape{ctx->cells_per_thread, ctx->block_threads, ctx->rows_per_block, ctx->l2_policy};
    save_tune_file();
    return cudaSuccess;
}

unsigned d2q9_take_pipe_status(lbm_ctx *ctx) {
    if (!ctx->pipe_status_d) return 0;
    unsigned h = 0;
    if (cudaMemcpyAsync(&h, ctx->pipe_status_d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        return ~0u;
    if (h && (cudaMemsetAsync(ctx->pipe_status_d, 0, sizeof(unsigned), ctx->stream) != cudaSuccess ||
              cudaStreamSynchronize(ctx->stream) != cudaSuccess))
        return ~0u;
    return h;
}

cudaError_t d2q9_step(lbm_ctx *ctx, int nsteps) {
    return dispatch(ctx->desc.dtype, [&](auto tag) { return launch_step<decltype(tag)>(ctx, nsteps); });
}

cudaError_t d2q9_moments(lbm_ctx *ctx, float *rho_d, float *ux_d, float *uy_d) {
    D2Q9Params prm = d2q9_params(ctx->desc);
    return dispatch(ctx->desc.dtype, [&](auto tag) {
        using S = decltype(tag);
        moments_kernel<S><<<row_grid(ctx, 256), 256, 0, ctx->stream>>>(
            static_cast<const S *>(ctx->f[ctx->cur]), ctx->links_d, ctx->desc.nx, ctx->desc.ny, ctx->pitch,
            ctx->plane, ctx->desc.periodic, prm, rho_d, ux_d, uy_d);
        return cudaGetLastError();
    });
}

cudaError_t d2q9_conservation(lbm_ctx *ctx, double *out_d) {
    const int nblocks = 512;
    return dispatch(ctx->desc.dtype, [&](auto tag) {
        using S = decltype(tag);
        conservation_kernel<S><<<nblocks, 256, 0, ctx->stream>>>(static_cast<const S *>(ctx->f[ctx->cur]),
                                                                 ctx->links_d, ctx->desc.nx, ctx->desc.ny,
                                                                 ctx->pitch, ctx->plane, ctx->scratch.partials);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        return finalize_sums(ctx->stream, ctx->scratch.partials, nblocks, 3, out_d);
    });
}

cudaError_t d2q9_load(lbm_ctx *ctx, const void *src_d, int src_dtype, int aos) {
    return dispatch(ctx->desc.dtype, [&](auto tag) {
        using S = decltype(tag);
        S *a = static_cast<S *>(ctx->f[0]), *b = static_cast<S *>(ctx->f[1]);
        if (aos || src_dtype == LBM_F32)
            load_kernel<S, float><<<row_grid(ctx, 128), 128, 0, ctx->stream>>>(
                a, b, static_cast<const float *>(src_d), ctx->desc.nx, ctx->desc.ny, ctx->pitch, ctx->plane, aos);
        else
            load_kernel<S, double><<<row_grid(ctx, 128), 128, 0, ctx->stream>>>(
                a, b, static_cast<const double *>(src_d), ctx->desc.nx, ctx->desc.ny, ctx->pitch, ctx->plane, aos);
        return cudaGetLastError();
    });
}

cudaError_t d2q9_store(lbm_ctx *ctx, void *dst_d, int dst_dtype, int aos) {
    return dispatch(ctx->desc.dtype, [&](auto tag) {
        using S = decltype(tag);
        const S *src = static_cast<const S *>(ctx->f[ctx->cur]);
        if (aos || dst_dtype == LBM_F32)
            store_kernel<S, float><<<row_grid(ctx, 128), 128, 0, ctx->stream>>>(
                src, static_cast<float *>(dst_d), ctx->desc.nx, ctx->desc.ny, ctx->pitch, ctx->plane, aos,
                ctx->flags_set ? ctx->flags_d : nullptr);
        else
            store_kernel<S, double><<<row_grid(ctx, 128), 128, 0, ctx->stream>>>(
                src, static_cast<double *>(dst_d), ctx->desc.nx, ctx->desc.ny, ctx->pitch, ctx->plane, aos,
                nullptr);
        return cudaGetLastError();
    });
}

}  // namespace lbm
