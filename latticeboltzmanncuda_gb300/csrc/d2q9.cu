// D2Q9 kernels: fused pull step (streaming + half-way bounce-back + moving walls + periodic wrap +
// BGK collision + Guo forcing in one pass: one read and one write of the nine populations per
// cell update), link-word construction, equilibrium initialisation, moments, FP64 conservation
// sums and host-layout conversion.
//
// Storage: structure of arrays, plane q holds population q of all cells, rows padded to `pitch`
// elements (a multiple of 32) so each row starts 128-byte aligned in FP32.  Populations are
// stored shifted, g_q = f_q - w_q, in FP32 / FP16 / BF16 (arithmetic in FP32) or FP64 (the GPU
// oracle).  Two buffers (A/B): step n reads f[cur] and writes f[cur ^ 1].
//
// Population order: 0:(0,0) 1:(1,0) 2:(0,1) 3:(-1,0) 4:(0,-1) 5:(1,1) 6:(-1,1) 7:(-1,-1) 8:(1,-1).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "lbm_internal.h"
#include "d2q9_core.cuh"
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
__global__ void build_links_kernel(const uint8_t *__restrict__ flags, uint16_t *__restrict__ links,
                                   int nx, int ny, int64_t pitch, int periodic) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= nx) return;
    int64_t c = (int64_t)y * pitch + x;
    if (flags[(int64_t)y * nx + x] != 0) {
        links[c] = LINK_SOLID;
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
// fused step, one thread per cell
// ------------------------------------------------------------------------------------------------
template <class S, bool FORCE>
__global__ void __launch_bounds__(256) step_kernel(const S *__restrict__ src, S *__restrict__ dst,
                                                   const uint16_t *__restrict__ links, int nx, int ny,
                                                   int64_t pitch, int64_t plane, int periodic,
                                                   D2Q9Params prm) {
    using R = typename d2q9::Store<S>::R;
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= nx) return;
    int64_t c = (int64_t)y * pitch + x;
    uint16_t L = __ldg(links + c);
    if (L == LINK_SOLID) return;
    R g[9];
    d2q9::gather<S>(src, L, x, y, nx, ny, pitch, plane, periodic, d2q9::wall_u<R>(prm), g);
    d2q9::collide<R, FORCE>(g, d2q9::omega<R>(prm), d2q9::force<R>(prm));
#pragma unroll
    for (int q = 0; q < 9; ++q) d2q9::Store<S>::st(dst + q * plane + c, g[q]);
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
        R g[9];
        d2q9::gather<S>(src, L, x, y, nx, ny, pitch, plane, periodic, d2q9::wall_u<R>(prm), g);
        R drho, mx, my;
        d2q9::moments(g, drho, mx, my);
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
    R g[9];
    d2q9::equilibrium_shifted(r - (R)1, r, u, v, g);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        d2q9::Store<S>::st(a + q * plane + c, g[q]);
        d2q9::Store<S>::st(b + q * plane + c, g[q]);
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
        for (int q = 0; q < 9; ++q) g[q] = (double)d2q9::Store<S>::ld(src + q * plane + c);
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
        d2q9::Store<S>::st(a + q * plane + c, g);
        d2q9::Store<S>::st(b + q * plane + c, g);
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
        for (int q = 0; q < 9; ++q) f[aos_slot(q)] = (float)(d2q9::Store<S>::ld(src + q * plane + c) + d2q9::w<R>(q));
        uint8_t fl = flags ? flags[(int64_t)y * nx + x] : 0;
        rec[120] = 0;        // isReflected
        rec[121] = fl != 0;  // isInternal: solid cell
        *reinterpret_cast<unsigned long long *>(rec + 128) = 0ull;
        *reinterpret_cast<unsigned long long *>(rec + 136) = 0ull;
    } else {
#pragma unroll
        for (int q = 0; q < 9; ++q)
            host[q * n + (int64_t)y * nx + x] = (H)(d2q9::Store<S>::ld(src + q * plane + c) + d2q9::w<R>(q));
    }
}

template <class S>
cudaError_t launch_step(lbm_ctx *ctx, int nsteps) {
    const lbm_desc &d = ctx->desc;
    D2Q9Params prm = d2q9_params(d);
    bool force = prm.fx != 0.0f || prm.fy != 0.0f;
    dim3 block(ctx->block_threads);
    dim3 grid((unsigned)((d.nx + block.x - 1) / block.x), (unsigned)d.ny);
    for (int s = 0; s < nsteps; ++s) {
        const S *src = static_cast<const S *>(ctx->f[ctx->cur]);
        S *dst = static_cast<S *>(ctx->f[ctx->cur ^ 1]);
        if (force)
            step_kernel<S, true><<<grid, block, 0, ctx->stream>>>(src, dst, ctx->links_d, d.nx, d.ny, ctx->pitch,
                                                                   ctx->plane, d.periodic, prm);
        else
            step_kernel<S, false><<<grid, block, 0, ctx->stream>>>(src, dst, ctx->links_d, d.nx, d.ny, ctx->pitch,
                                                                    ctx->plane, d.periodic, prm);
        ctx->cur ^= 1;
    }
    return cudaGetLastError();
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

cudaError_t d2q9_build_links(lbm_ctx *ctx) {
    const lbm_desc &d = ctx->desc;
    build_links_kernel<<<row_grid(ctx, 256), 256, 0, ctx->stream>>>(ctx->flags_d, ctx->links_d, d.nx, d.ny,
                                                                    ctx->pitch, d.periodic);
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
