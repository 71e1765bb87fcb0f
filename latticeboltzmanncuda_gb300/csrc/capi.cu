// C ABI entry points (include/lbm_capi.h): argument checks, context life cycle, host <-> device
// staging, and the host-side construction of the D3Q27_REF gather lists.
#include <algorithm>
#include <cstring>
#include <string>
#include <tuple>
#include <vector>

#include "lbm_internal.h"

using namespace lbm;

namespace lbm {
const char *thread_error();
}

namespace {

constexpr uint8_t F_GATHER = 8;

// D3Q27 directions (SimCalcFuncs.cu:12), host copy for the gather-list construction
constexpr auto &C27 = lbm::kD3Q27;

#define CHECK_CTX(ctx)                                                              \
    do {                                                                            \
        if (!(ctx)) return set_thread_error(LBM_ERR_INVALID, "null context");       \
    } while (0)

#define CUDA_TRY(ctx, call, what)                              \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

lbm_status use_device(lbm_ctx *ctx) {
    CUDA_TRY(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
    return LBM_OK;
}

size_t dtype_size(int dtype) {
    switch (dtype) {
        case LBM_F32: return 4;
        case LBM_F16S:
        case LBM_BF16S: return 2;
        case LBM_F64: return 8;
    }
    return 0;
}

lbm_status ensure_staging(lbm_ctx *ctx, size_t bytes) {
    if (ctx->staging_bytes >= bytes) return LBM_OK;
    if (ctx->staging) {
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "synchronize before staging resize");
    }
    dfree(ctx, ctx->staging, ctx->staging_bytes);
    ctx->staging = nullptr;
    ctx->staging_bytes = 0;
    lbm_status s = dalloc(ctx, &ctx->staging, bytes, "host-layout staging");
    if (s == LBM_OK) ctx->staging_bytes = bytes;
    return s;
}

lbm_status sync(lbm_ctx *ctx, const char *what) {
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), what);
    if (ctx->pipe_used) {
        ctx->pipe_used = false;
        const unsigned bits = d2q9_take_pipe_status(ctx);
        if (bits)
            return fail(ctx, LBM_ERR_TIMEOUT,
                        std::string(what) + ": a bounded wait of the D2Q9 bulk-copy pipeline gave up; the populations "
                                            "of the steps since the last synchronisation are not valid");
    }
    return LBM_OK;
}

// Rebuild the D3Q27_REF gather lists from the host tables and flags and upload the flag bytes.
lbm_status d3_prepare(lbm_ctx *ctx) {
    if (!ctx->d3_dirty) return LBM_OK;
    const int X = ctx->desc.nx, Y = ctx->desc.ny, Z = ctx->desc.nz;
    std::vector<uint8_t> fl(ctx->flags_h);
    for (auto &b : fl) b &= (uint8_t)(LBM_INTERNAL | LBM_REFLECTED | LBM_SOURCE);

    struct Ent {
        int32_t tgt;
        GatherEntry e;
    };
    std::vector<Ent> ents;
    for (const auto &tr : ctx->tables_h) {
        const int32_t yc = tr.first;
        if (!(fl[yc] & LBM_REFLECTED)) continue;  // SimCalcFuncs.cu:162
        const ReflRecord &r = tr.second;
        const int z = yc % Z, t0 = yc / Z, y = t0 % Y, x = t0 / Y;
        for (int s = 1; s < 81; ++s) {  // slot 0 is never read (SimCalcFuncs.cu:164)
            const int d = refl_dir(r, s);
            if (d == 0) continue;
            if (d > 26)
                return fail(ctx, LBM_ERR_INVALID, "reflection table of cell " + std::to_string(yc) + " slot " +
                                                      std::to_string(s) + " names direction " + std::to_string(d) +
                                                      " (valid: 1..26)");
            const int tx = x + C27[d][0], ty = y + C27[d][1], tz = z + C27[d][2];
            if (tx < 0 || ty < 0 || tz < 0 || tx >= X || ty >= Y || tz >= Z) continue;  // SimCalcFuncs.cu:175
            const int p = s / 3;
            const int sx = x - C27[p][0], sy = y - C27[p][1], sz = z - C27[p][2];
            const bool in = sx >= 0 && sy >= 0 && sz >= 0 && sx < X && sy < Y && sz < Z;
            Ent en;
            en.tgt = tz + Z * (ty + Y * tx);
            en.e.src_cell = yc;
            en.e.src_stream = in ? (int32_t)(sz + Z * (sy + Y * sx)) : -1;
            en.e.w = r.w[s];
            en.e.src_pop = (uint8_t)p;
            en.e.dst_pop = (uint8_t)d;
            en.e.slot = (uint8_t)s;
            en.e.pad = 0;
            ents.push_back(en);
        }
    }
    std::stable_sort(ents.begin(), ents.end(), [](const Ent &a, const Ent &b) {
        return std::make_tuple(a.tgt, a.e.src_cell, a.e.slot) < std::make_tuple(b.tgt, b.e.src_cell, b.e.slot);
    });
    std::vector<int32_t> tgt, off;
    std::vector<GatherEntry> flat;
    flat.reserve(ents.size());
    for (size_t i = 0; i < ents.size(); ++i) {
        if (i == 0 || ents[i].tgt != ents[i - 1].tgt) {
            tgt.push_back(ents[i].tgt);
            off.push_back((int32_t)i);
            fl[ents[i].tgt] |= F_GATHER;
        }
        flat.push_back(ents[i].e);
    }
    off.push_back((int32_t)ents.size());

    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "synchronize before table upload");
    dfree(ctx, ctx->tgt_cells_d, ctx->ntgt * sizeof(int32_t));
    dfree(ctx, ctx->tgt_off_d, (ctx->ntgt + 1) * sizeof(int32_t));
    dfree(ctx, ctx->entries_d, ctx->nent * sizeof(GatherEntry));
    dfree(ctx, ctx->gathered_d, ctx->ntgt * 27 * sizeof(float));
    dfree(ctx, ctx->tgt_index_d, ctx->ntgt ? (size_t)ctx->cells * sizeof(int32_t) : 0);
    dfree(ctx, ctx->gather_done_d, ctx->ntgt ? 16 : 0);
    ctx->gather_done_d = nullptr;
    ctx->gathered_d = nullptr;
    ctx->tgt_index_d = nullptr;
    ctx->tgt_cells_d = nullptr;
    ctx->tgt_off_d = nullptr;
    ctx->entries_d = nullptr;
    ctx->ntgt = (int64_t)tgt.size();
    ctx->nent = (int64_t)flat.size();
    if (ctx->ntgt) {
        lbm_status s;
        if ((s = dalloc(ctx, (void **)&ctx->tgt_cells_d, tgt.size() * sizeof(int32_t), "gather targets")) != LBM_OK) return s;
        if ((s = dalloc(ctx, (void **)&ctx->tgt_off_d, off.size() * sizeof(int32_t), "gather offsets")) != LBM_OK) return s;
        if ((s = dalloc(ctx, (void **)&ctx->entries_d, flat.size() * sizeof(GatherEntry), "gather entries")) != LBM_OK) return s;
        CUDA_TRY(ctx, cudaMemcpy(ctx->tgt_cells_d, tgt.data(), tgt.size() * sizeof(int32_t), cudaMemcpyHostToDevice), "upload gather targets");
        CUDA_TRY(ctx, cudaMemcpy(ctx->tgt_off_d, off.data(), off.size() * sizeof(int32_t), cudaMemcpyHostToDevice), "upload gather offsets");
        CUDA_TRY(ctx, cudaMemcpy(ctx->entries_d, flat.data(), flat.size() * sizeof(GatherEntry), cudaMemcpyHostToDevice), "upload gather entries");
        if ((s = dalloc(ctx, (void **)&ctx->gathered_d, tgt.size() * 27 * sizeof(float), "gathered populations")) != LBM_OK)
            return s;
        if ((s = dalloc(ctx, (void **)&ctx->tgt_index_d, (size_t)ctx->cells * sizeof(int32_t), "target index")) != LBM_OK)
            return s;
        if ((s = dalloc(ctx, (void **)&ctx->gather_done_d, 16, "gather block counter")) != LBM_OK) return s;
        CUDA_TRY(ctx, cudaMemset(ctx->gather_done_d, 0, 16), "clear gather block counter");
        std::vector<int32_t> index((size_t)ctx->cells, -1);
        for (size_t k = 0; k < tgt.size(); ++k) index[(size_t)tgt[k]] = (int32_t)k;
        CUDA_TRY(ctx, cudaMemcpy(ctx->tgt_index_d, index.data(), index.size() * sizeof(int32_t), cudaMemcpyHostToDevice),
                 "upload target index");
        const size_t nblocks = d3q27_gather_blocks(ctx->ntgt);
        if ((s = ensure_scratch(ctx, std::max<size_t>(nblocks * 3, 512 * 4))) != LBM_OK) return s;
    }
    CUDA_TRY(ctx, cudaMemcpy(ctx->flags_d, fl.data(), fl.size(), cudaMemcpyHostToDevice), "upload flags");
    ctx->d3_dirty = false;
    return LBM_OK;
}

lbm_status validate_desc(const lbm_desc *d) {
    if (!d) return set_thread_error(LBM_ERR_INVALID, "null descriptor");
    if (d->mode != LBM_D2Q9 && d->mode != LBM_D3Q27_REF)
        return set_thread_error(LBM_ERR_INVALID, "mode must be LBM_D2Q9 or LBM_D3Q27_REF");
    if (dtype_size(d->dtype) == 0) return set_thread_error(LBM_ERR_INVALID, "unknown dtype");
    if (d->nx < 1 || d->ny < 1 || d->nz < 1) return set_thread_error(LBM_ERR_INVALID, "dimensions must be >= 1");
    const int64_t cells = (int64_t)d->nx * d->ny * d->nz;
    if (cells > (int64_t)INT32_MAX) return set_thread_error(LBM_ERR_INVALID, "more than 2^31-1 cells");
    if (!(d->tau == d->tau) || d->tau == 0.0f) return set_thread_error(LBM_ERR_INVALID, "tau must be non-zero");
    if (d->mode == LBM_D2Q9) {
        if (d->nz != 1) return set_thread_error(LBM_ERR_INVALID, "D2Q9 needs nz == 1");
        if (!(d->tau > 0.5f)) return set_thread_error(LBM_ERR_INVALID, "D2Q9 needs tau > 0.5");
        if (d->periodic < 0 || d->periodic > 3) return set_thread_error(LBM_ERR_INVALID, "periodic must be 0..3");
    } else {
        if (d->dtype != LBM_F32) return set_thread_error(LBM_ERR_UNSUPPORTED, "D3Q27_REF stores FP32 populations only");
        if (d->order != LBM_ORDER_STREAM_COLLIDE && d->order != LBM_ORDER_CLI)
            return set_thread_error(LBM_ERR_INVALID, "unknown D3Q27_REF step order");
        if (d->force_mode != LBM_FORCE_REFERENCE && d->force_mode != LBM_FORCE_MOMENTUM_EXCHANGE)
            return set_thread_error(LBM_ERR_INVALID, "unknown force_mode");
    }
    return LBM_OK;
}

}  // namespace

extern "C" {

LBM_API void lbm_desc_init(lbm_desc *d) {
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
    d->mode = LBM_D2Q9;
    d->dtype = LBM_F32;
    d->nx = d->ny = d->nz = 1;
    d->tau = 1.0f;
    d->order = LBM_ORDER_STREAM_COLLIDE;
    d->force_mode = LBM_FORCE_REFERENCE;
}

LBM_API const char *lbm_status_string(lbm_status s) {
    switch (s) {
        case LBM_OK: return "ok";
        case LBM_ERR_INVALID: return "invalid argument";
        case LBM_ERR_CUDA: return "CUDA error";
        case LBM_ERR_OOM: return "out of device memory";
        case LBM_ERR_UNSUPPORTED: return "unsupported";
        case LBM_ERR_STATE: return "bad state";
        case LBM_ERR_BUDGET: return "over memory budget";
        case LBM_ERR_TIMEOUT: return "timeout";
    }
    return "unknown status";
}

LBM_API const char *lbm_last_error(const lbm_ctx *ctx) { return ctx ? ctx->err.c_str() : lbm::thread_error(); }

LBM_API lbm_status lbm_create(const lbm_desc *desc, lbm_ctx **out) {
    if (!out) return set_thread_error(LBM_ERR_INVALID, "null output pointer");
    *out = nullptr;
    lbm_status st = validate_desc(desc);
    if (st != LBM_OK) return st;
    lbm_ctx *ctx = new lbm_ctx();
    ctx->desc = *desc;
    ctx->device = desc->device;
    auto bail = [&](lbm_status s) {
        lbm_destroy(ctx);
        return s;
    };
    if ((st = use_device(ctx)) != LBM_OK) return bail(set_thread_error(st, ctx->err));
    if (desc->stream) {
        ctx->stream = static_cast<cudaStream_t>(desc->stream);
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "cudaStreamCreate"));
        ctx->own_stream = true;
    }
    const lbm_desc &d = ctx->desc;
    ctx->cells = (int64_t)d.nx * d.ny * d.nz;
    void *p = nullptr;
    if ((st = dalloc(ctx, &p, 16 * sizeof(double), "result buffer")) != LBM_OK) return bail(set_thread_error(st, ctx->err));
    ctx->result_d = static_cast<double *>(p);
    if ((st = ensure_scratch(ctx, 512 * 4)) != LBM_OK) return bail(set_thread_error(st, ctx->err));
    if (d.mode == LBM_D2Q9) {
        ctx->q = 9;
        ctx->elem = dtype_size(d.dtype);
        ctx->pitch = ((int64_t)d.nx + 31) / 32 * 32;
        ctx->plane = ctx->pitch * d.ny;
        for (int b = 0; b < 2; ++b)
            if ((st = dalloc(ctx, &ctx->f[b], (size_t)ctx->plane * 9 * ctx->elem, "populations")) != LBM_OK)
                return bail(set_thread_error(st, ctx->err));
        if ((st = dalloc(ctx, (void **)&ctx->flags_d, (size_t)ctx->cells, "flags")) != LBM_OK)
            return bail(set_thread_error(st, ctx->err));
        if ((st = dalloc(ctx, (void **)&ctx->links_d, (size_t)ctx->plane * sizeof(uint16_t), "links")) != LBM_OK)
            return bail(set_thread_error(st, ctx->err));
        if ((st = dalloc(ctx, (void **)&ctx->pipe_status_d, 16, "pipeline status")) != LBM_OK)
            return bail(set_thread_error(st, ctx->err));
        cudaError_t e = cudaMemsetAsync(ctx->flags_d, 0, (size_t)ctx->cells, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->pipe_status_d, 0, 16, ctx->stream);
        // link words of the row padding stay 0 (the vectorised step reads them)
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->links_d, 0, (size_t)ctx->plane * sizeof(uint16_t), ctx->stream);
        if (e == cudaSuccess) e = d2q9_build_links(ctx);
        if (e == cudaSuccess) e = d2q9_init_equilibrium(ctx, nullptr, nullptr, nullptr);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "D2Q9 initialisation"));
        ctx->flags_set = true;
    } else {
        ctx->q = 27;
        ctx->elem = 4;
        ctx->pitch = ctx->cells;
        ctx->plane = ctx->cells;
        for (int b = 0; b < 2; ++b) {
            if ((st = dalloc(ctx, &ctx->f[b], (size_t)ctx->plane * 27 * 4, "populations")) != LBM_OK)
                return bail(set_thread_error(st, ctx->err));
            cudaError_t e = cudaMemsetAsync(ctx->f[b], 0, (size_t)ctx->plane * 27 * 4, ctx->stream);
            if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "clear populations"));
        }
        if ((st = dalloc(ctx, (void **)&ctx->flags_d, (size_t)ctx->cells, "flags")) != LBM_OK)
            return bail(set_thread_error(st, ctx->err));
        if ((st = dalloc(ctx, (void **)&ctx->induced_d, 27 * sizeof(float), "induced flow")) != LBM_OK)
            return bail(set_thread_error(st, ctx->err));
        if ((st = dalloc(ctx, (void **)&ctx->force_acc_d, 4 * sizeof(double), "force")) != LBM_OK)
            return bail(set_thread_error(st, ctx->err));
        cudaError_t e = cudaMemsetAsync(ctx->force_acc_d, 0, 4 * sizeof(double), ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->induced_d, 0, 27 * sizeof(float), ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "D3Q27 initialisation"));
        ctx->flags_h.assign((size_t)ctx->cells, 0);
        ctx->d3_dirty = true;
        ctx->flags_set = true;
        if ((st = d3_prepare(ctx)) != LBM_OK) return bail(set_thread_error(st, ctx->err));
    }
    *out = ctx;
    return LBM_OK;
}

LBM_API lbm_status lbm_destroy(lbm_ctx *ctx) {
    if (!ctx) return LBM_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (int b = 0; b < 2; ++b) cudaFree(ctx->f[b]);
    cudaFree(ctx->flags_d);
    cudaFree(ctx->links_d);
    cudaFree(ctx->pipe_status_d);
    cudaFree(ctx->tgt_cells_d);
    cudaFree(ctx->tgt_off_d);
    cudaFree(ctx->entries_d);
    cudaFree(ctx->gathered_d);
    cudaFree(ctx->tgt_index_d);
    cudaFree(ctx->gather_done_d);
    cudaFree(ctx->induced_d);
    cudaFree(ctx->force_acc_d);
    cudaFree(ctx->scratch.partials);
    cudaFree(ctx->result_d);
    cudaFree(ctx->staging);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return LBM_OK;
}

LBM_API lbm_status lbm_get_info(lbm_ctx *ctx, lbm_info *out) {
    CHECK_CTX(ctx);
    if (!out) return fail(ctx, LBM_ERR_INVALID, "null output");
    out->cells = ctx->cells;
    out->fluid_cells = ctx->desc.mode == LBM_D2Q9 ? ctx->fluid_cells : ctx->cells;
    out->row_pitch = ctx->pitch;
    out->state_bytes = (int64_t)(2 * (size_t)ctx->plane * ctx->q * ctx->elem);
    out->device_bytes = (int64_t)ctx->device_bytes;
    out->bytes_per_update = (int64_t)(2 * ctx->q * ctx->elem);
    out->steps_done = ctx->steps_done;
    out->block_threads = ctx->block_threads;
    out->cells_per_thread = ctx->cells_per_thread;
    out->rows_per_block = ctx->rows_per_block;
    out->tuned = ctx->tuned ? 1 : 0;
    out->l2_policy = ctx->l2_policy;
    return LBM_OK;
}

LBM_API lbm_status lbm_get_stream(lbm_ctx *ctx, void **stream) {
    CHECK_CTX(ctx);
    if (!stream) return fail(ctx, LBM_ERR_INVALID, "null output");
    *stream = ctx->stream;
    return LBM_OK;
}

LBM_API lbm_status lbm_synchronize(lbm_ctx *ctx) {
    CHECK_CTX(ctx);
    return sync(ctx, "cudaStreamSynchronize");
}

LBM_API lbm_status lbm_set_params(lbm_ctx *ctx, float tau, const float body_force[3], const float wall_velocity[3]) {
    CHECK_CTX(ctx);
    lbm_desc d = ctx->desc;
    d.tau = tau;
    if (body_force) std::memcpy(d.body_force, body_force, sizeof(d.body_force));
    if (wall_velocity) std::memcpy(d.wall_velocity, wall_velocity, sizeof(d.wall_velocity));
    lbm_status s = validate_desc(&d);
    if (s != LBM_OK) return fail(ctx, s, lbm::thread_error());
    ctx->desc = d;
    return LBM_OK;
}

LBM_API lbm_status lbm_set_flags(lbm_ctx *ctx, const uint8_t *host_flags) {
    CHECK_CTX(ctx);
    if (!host_flags) return fail(ctx, LBM_ERR_INVALID, "null flags");
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    const size_t n = (size_t)ctx->cells;
    if (ctx->desc.mode == LBM_D2Q9) {
        for (size_t i = 0; i < n; ++i)
            if (host_flags[i] > LBM_MOVING_WALL)
                return fail(ctx, LBM_ERR_INVALID, "D2Q9 flag " + std::to_string(host_flags[i]) + " at cell " +
                                                      std::to_string(i) + " (valid: 0 fluid, 1 wall, 2 moving wall)");
        CUDA_TRY(ctx, cudaMemcpyAsync(ctx->flags_d, host_flags, n, cudaMemcpyHostToDevice, ctx->stream), "upload flags");
        CUDA_TRY(ctx, d2q9_build_links(ctx), "build link words");
    } else {
        for (size_t i = 0; i < n; ++i)
            if (host_flags[i] & ~(LBM_INTERNAL | LBM_REFLECTED | LBM_SOURCE))
                return fail(ctx, LBM_ERR_INVALID, "D3Q27_REF flag bits must be within LBM_INTERNAL|LBM_REFLECTED|LBM_SOURCE");
        std::memcpy(ctx->flags_h.data(), host_flags, n);
        ctx->d3_dirty = true;
        if ((st = d3_prepare(ctx)) != LBM_OK) return st;
    }
    ctx->flags_set = true;
    return LBM_OK;
}

LBM_API lbm_status lbm_get_flags(lbm_ctx *ctx, uint8_t *host_flags) {
    CHECK_CTX(ctx);
    if (!host_flags) return fail(ctx, LBM_ERR_INVALID, "null flags");
    if (ctx->desc.mode == LBM_D3Q27_REF) {
        for (size_t i = 0; i < ctx->flags_h.size(); ++i) host_flags[i] = ctx->flags_h[i];
        return LBM_OK;
    }
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    CUDA_TRY(ctx, cudaMemcpyAsync(host_flags, ctx->flags_d, (size_t)ctx->cells, cudaMemcpyDeviceToHost, ctx->stream),
             "download flags");
    return sync(ctx, "download flags");
}

LBM_API lbm_status lbm_init_equilibrium(lbm_ctx *ctx, const float *rho, const float *ux, const float *uy) {
    CHECK_CTX(ctx);
    if (ctx->desc.mode != LBM_D2Q9) return fail(ctx, LBM_ERR_UNSUPPORTED, "lbm_init_equilibrium is D2Q9 only");
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    const size_t n = (size_t)ctx->cells;
    if ((st = ensure_staging(ctx, 3 * n * sizeof(float))) != LBM_OK) return st;
    float *base = static_cast<float *>(ctx->staging);
    const float *src[3] = {rho, ux, uy};
    float *dev[3] = {nullptr, nullptr, nullptr};
    for (int k = 0; k < 3; ++k) {
        if (!src[k]) continue;
        dev[k] = base + k * n;
        CUDA_TRY(ctx, cudaMemcpyAsync(dev[k], src[k], n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
                 "upload initial fields");
    }
    CUDA_TRY(ctx, d2q9_init_equilibrium(ctx, dev[0], dev[1], dev[2]), "equilibrium kernel");
    return sync(ctx, "equilibrium");
}

LBM_API lbm_status lbm_load_populations(lbm_ctx *ctx, const void *host, int32_t host_dtype) {
    CHECK_CTX(ctx);
    if (!host) return fail(ctx, LBM_ERR_INVALID, "null host buffer");
    if (host_dtype != LBM_F32 && host_dtype != LBM_F64) return fail(ctx, LBM_ERR_INVALID, "host dtype must be LBM_F32 or LBM_F64");
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    const size_t bytes = (size_t)ctx->cells * ctx->q * dtype_size(host_dtype);
    if ((st = ensure_staging(ctx, bytes)) != LBM_OK) return st;
    CUDA_TRY(ctx, cudaMemcpyAsync(ctx->staging, host, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload populations");
    CUDA_TRY(ctx, ctx->desc.mode == LBM_D2Q9 ? d2q9_load(ctx, ctx->staging, host_dtype, 0)
                                            : d3q27_load(ctx, ctx->staging, host_dtype, 0),
             "load kernel");
    return sync(ctx, "load populations");
}

LBM_API lbm_status lbm_retrieve_populations(lbm_ctx *ctx, void *host, int32_t host_dtype) {
    CHECK_CTX(ctx);
    if (!host) return fail(ctx, LBM_ERR_INVALID, "null host buffer");
    if (host_dtype != LBM_F32 && host_dtype != LBM_F64) return fail(ctx, LBM_ERR_INVALID, "host dtype must be LBM_F32 or LBM_F64");
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    const size_t bytes = (size_t)ctx->cells * ctx->q * dtype_size(host_dtype);
    if ((st = ensure_staging(ctx, bytes)) != LBM_OK) return st;
    CUDA_TRY(ctx, ctx->desc.mode == LBM_D2Q9 ? d2q9_store(ctx, ctx->staging, host_dtype, 0)
                                            : d3q27_store(ctx, ctx->staging, host_dtype, 0),
             "store kernel");
    CUDA_TRY(ctx, cudaMemcpyAsync(host, ctx->staging, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download populations");
    return sync(ctx, "retrieve populations");
}

LBM_API lbm_status lbm_load_aos(lbm_ctx *ctx, const void *host_points, int64_t count) {
    CHECK_CTX(ctx);
    if (!host_points) return fail(ctx, LBM_ERR_INVALID, "null host buffer");
    if (count != ctx->cells)
        return fail(ctx, LBM_ERR_INVALID, "record count " + std::to_string(count) + " != cells " + std::to_string(ctx->cells));
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    const size_t bytes = (size_t)count * 144;
    if ((st = ensure_staging(ctx, bytes)) != LBM_OK) return st;
    CUDA_TRY(ctx, cudaMemcpyAsync(ctx->staging, host_points, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload records");
    if (ctx->desc.mode == LBM_D2Q9) {
        CUDA_TRY(ctx, d2q9_load(ctx, ctx->staging, LBM_F32, 1), "load kernel");
    } else {
        CUDA_TRY(ctx, d3q27_load(ctx, ctx->staging, LBM_F32, 1), "load kernel");
        // LatticePoint::isReflected at byte 120, isInternal at byte 121 (LatticePoint.h:13-14)
        const unsigned char *rec = static_cast<const unsigned char *>(host_points);
        for (int64_t c = 0; c < count; ++c) {
            uint8_t f = ctx->flags_h[(size_t)c] & LBM_SOURCE;
            if (rec[c * 144 + 121]) f |= LBM_INTERNAL;
            if (rec[c * 144 + 120]) f |= LBM_REFLECTED;
            ctx->flags_h[(size_t)c] = f;
        }
        ctx->d3_dirty = true;
        if ((st = sync(ctx, "load records")) != LBM_OK) return st;
        return d3_prepare(ctx);
    }
    return sync(ctx, "load records");
}

LBM_API lbm_status lbm_retrieve_aos(lbm_ctx *ctx, void *host_points, int64_t count) {
    CHECK_CTX(ctx);
    if (!host_points) return fail(ctx, LBM_ERR_INVALID, "null host buffer");
    if (count != ctx->cells)
        return fail(ctx, LBM_ERR_INVALID, "record count " + std::to_string(count) + " != cells " + std::to_string(ctx->cells));
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    if (ctx->desc.mode == LBM_D3Q27_REF && (st = d3_prepare(ctx)) != LBM_OK) return st;
    const size_t bytes = (size_t)count * 144;
    if ((st = ensure_staging(ctx, bytes)) != LBM_OK) return st;
    CUDA_TRY(ctx, ctx->desc.mode == LBM_D2Q9 ? d2q9_store(ctx, ctx->staging, LBM_F32, 1)
                                            : d3q27_store(ctx, ctx->staging, LBM_F32, 1),
             "store kernel");
    CUDA_TRY(ctx, cudaMemcpyAsync(host_points, ctx->staging, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download records");
    return sync(ctx, "retrieve records");
}

LBM_API lbm_status lbm_set_reflection_tables(lbm_ctx *ctx, int64_t count, const int32_t *cells, const void *records) {
    CHECK_CTX(ctx);
    if (ctx->desc.mode != LBM_D3Q27_REF) return fail(ctx, LBM_ERR_UNSUPPORTED, "reflection tables are D3Q27_REF only");
    if (count < 0 || (count > 0 && (!cells || !records))) return fail(ctx, LBM_ERR_INVALID, "bad table arguments");
    std::vector<std::pair<int32_t, ReflRecord>> t;
    t.reserve((size_t)count);
    std::vector<uint8_t> seen((size_t)ctx->cells, 0);
    const ReflRecord *r = static_cast<const ReflRecord *>(records);
    for (int64_t i = 0; i < count; ++i) {
        if (cells[i] < 0 || cells[i] >= ctx->cells)
            return fail(ctx, LBM_ERR_INVALID, "table cell index " + std::to_string(cells[i]) + " out of range");
        if (seen[(size_t)cells[i]]++)
            return fail(ctx, LBM_ERR_INVALID, "two tables for cell " + std::to_string(cells[i]));
        t.emplace_back(cells[i], r[i]);
    }
    ctx->tables_h.swap(t);
    ctx->d3_dirty = true;
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    return d3_prepare(ctx);
}

LBM_API lbm_status lbm_set_flow(lbm_ctx *ctx, const uint8_t *mask, const float *induced) {
    CHECK_CTX(ctx);
    if (ctx->desc.mode != LBM_D3Q27_REF) return fail(ctx, LBM_ERR_UNSUPPORTED, "flow sources are D3Q27_REF only");
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    if (mask) {
        for (size_t c = 0; c < ctx->flags_h.size(); ++c)
            ctx->flags_h[c] = (uint8_t)((ctx->flags_h[c] & ~LBM_SOURCE) | (mask[c] ? LBM_SOURCE : 0));
        ctx->d3_dirty = true;
        if ((st = d3_prepare(ctx)) != LBM_OK) return st;
    }
    if (induced) {
        CUDA_TRY(ctx, cudaMemcpyAsync(ctx->induced_d, induced, 27 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
                 "upload induced flow");
        ctx->flow_on = true;
        return sync(ctx, "upload induced flow");
    }
    ctx->flow_on = false;
    return LBM_OK;
}

LBM_API lbm_status lbm_set_force(lbm_ctx *ctx, const float in[3], int32_t enabled) {
    CHECK_CTX(ctx);
    if (ctx->desc.mode != LBM_D3Q27_REF) return fail(ctx, LBM_ERR_UNSUPPORTED, "force accumulation is D3Q27_REF only");
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    double h[4] = {in ? in[0] : 0.0, in ? in[1] : 0.0, in ? in[2] : 0.0, 0.0};
    CUDA_TRY(ctx, cudaMemcpyAsync(ctx->force_acc_d, h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream), "upload force");
    ctx->force_on = enabled != 0;
    if (ctx->force_on && (st = ensure_scratch(ctx, std::max<size_t>(d3q27_gather_blocks(ctx->ntgt) * 3, 512 * 4))) != LBM_OK)
        return st;
    return sync(ctx, "upload force");
}

LBM_API lbm_status lbm_set_force_accumulation(lbm_ctx *ctx, int32_t enabled) {
    CHECK_CTX(ctx);
    if (ctx->desc.mode != LBM_D3Q27_REF) return fail(ctx, LBM_ERR_UNSUPPORTED, "force accumulation is D3Q27_REF only");
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    ctx->force_on = enabled != 0;
    if (ctx->force_on && (st = ensure_scratch(ctx, std::max<size_t>(d3q27_gather_blocks(ctx->ntgt) * 3, 512 * 4))) != LBM_OK)
        return st;
    return LBM_OK;
}

LBM_API int32_t lbm_force_accumulation(const lbm_ctx *ctx) { return ctx && ctx->force_on ? 1 : 0; }

LBM_API lbm_status lbm_get_force(lbm_ctx *ctx, float out[3]) {
    CHECK_CTX(ctx);
    if (!out) return fail(ctx, LBM_ERR_INVALID, "null output");
    if (ctx->desc.mode != LBM_D3Q27_REF) return fail(ctx, LBM_ERR_UNSUPPORTED, "force accumulation is D3Q27_REF only");
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    double h[4];
    CUDA_TRY(ctx, cudaMemcpyAsync(h, ctx->force_acc_d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream), "download force");
    if ((st = sync(ctx, "download force")) != LBM_OK) return st;
    for (int k = 0; k < 3; ++k) out[k] = (float)h[k];
    return LBM_OK;
}

LBM_API lbm_status lbm_step(lbm_ctx *ctx, int32_t nsteps) {
    CHECK_CTX(ctx);
    if (nsteps < 0) return fail(ctx, LBM_ERR_INVALID, "nsteps must be >= 0");
    if (nsteps == 0) return LBM_OK;
    NvtxRange range(ctx->desc.mode == LBM_D2Q9 ? "lbm_step d2q9" : "lbm_step d3q27_ref");
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    if (ctx->desc.mode == LBM_D2Q9) {
        CUDA_TRY(ctx, d2q9_step(ctx, nsteps), "D2Q9 step");
    } else {
        if ((st = d3_prepare(ctx)) != LBM_OK) return st;
        CUDA_TRY(ctx, d3q27_step(ctx, nsteps), "D3Q27 step");
    }
    ctx->steps_done += nsteps;
    return LBM_OK;
}

LBM_API lbm_status lbm_step_force_series(lbm_ctx *ctx, int32_t nsteps, float *host_series) {
    CHECK_CTX(ctx);
    if (ctx->desc.mode != LBM_D3Q27_REF) return fail(ctx, LBM_ERR_UNSUPPORTED, "force series are D3Q27_REF only");
    if (nsteps < 0 || (nsteps > 0 && !host_series)) return fail(ctx, LBM_ERR_INVALID, "bad nsteps or null series");
    if (nsteps == 0) return LBM_OK;
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    if ((st = d3_prepare(ctx)) != LBM_OK) return st;
    double *series_d = nullptr;
    const size_t bytes = (size_t)nsteps * 3 * sizeof(double);
    if ((st = dalloc(ctx, (void **)&series_d, bytes, "force series")) != LBM_OK) return st;
    std::vector<double> h((size_t)nsteps * 3);
    cudaError_t e = d3q27_step(ctx, nsteps, series_d);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), series_d, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dfree(ctx, series_d, bytes);
    if (e != cudaSuccess) return fail(ctx, e == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA,
                                      std::string("D3Q27 step with force series: ") + cudaGetErrorString(e));
    for (size_t i = 0; i < h.size(); ++i) host_series[i] = (float)h[i];
    ctx->steps_done += nsteps;
    return LBM_OK;
}

LBM_API lbm_status lbm_set_equilibrium_evaluation(lbm_ctx *ctx, int32_t mode) {
    CHECK_CTX(ctx);
    if (ctx->desc.mode != LBM_D3Q27_REF) return fail(ctx, LBM_ERR_UNSUPPORTED, "equilibrium evaluation is D3Q27_REF only");
    if (mode != LBM_EQ_FLOAT_FLOAT && mode != LBM_EQ_FP64 && mode != LBM_EQ_FP32)
        return fail(ctx, LBM_ERR_INVALID, "unknown equilibrium evaluation");
    ctx->eq_mode = mode;
    return LBM_OK;
}

LBM_API lbm_status lbm_d3q27_equilibrium_selftest(int64_t samples, uint64_t seed, int32_t device, int64_t out[2]) {
    if (samples < 0 || !out) return set_thread_error(LBM_ERR_INVALID, "lbm_d3q27_equilibrium_selftest: bad argument");
    cudaError_t e = cudaSetDevice(device);
    unsigned long long *d = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&d, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = d3q27_eq_selftest(samples, seed, d, nullptr);
    unsigned long long h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (e != cudaSuccess)
        return set_thread_error(LBM_ERR_CUDA, std::string("lbm_d3q27_equilibrium_selftest: ") + cudaGetErrorString(e));
    out[0] = (int64_t)h[0];
    out[1] = (int64_t)h[1];
    return LBM_OK;
}

LBM_API lbm_status lbm_d3q27_division_check(float tau, int32_t device, int64_t *mismatches) {
    if (!mismatches) return set_thread_error(LBM_ERR_INVALID, "lbm_d3q27_division_check: null output");
    cudaError_t e = cudaSetDevice(device);
    void *buf = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&buf, 16);
    if (e == cudaSuccess) e = cudaMemset(buf, 0, 16);
    if (e == cudaSuccess)
        e = d3q27_division_check(tau, reinterpret_cast<unsigned long long *>(static_cast<char *>(buf) + 8),
                                 static_cast<float *>(buf), nullptr);
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, static_cast<char *>(buf) + 8, sizeof(h), cudaMemcpyDeviceToHost);
    if (buf) cudaFree(buf);
    if (e != cudaSuccess)
        return set_thread_error(LBM_ERR_CUDA, std::string("lbm_d3q27_division_check: ") + cudaGetErrorString(e));
    *mismatches = (int64_t)h;
    return LBM_OK;
}

LBM_API lbm_status lbm_set_order(lbm_ctx *ctx, int32_t order) {
    CHECK_CTX(ctx);
    if (ctx->desc.mode != LBM_D3Q27_REF) return fail(ctx, LBM_ERR_UNSUPPORTED, "step orders are D3Q27_REF only");
    if (order != LBM_ORDER_STREAM_COLLIDE && order != LBM_ORDER_CLI) return fail(ctx, LBM_ERR_INVALID, "unknown step order");
    ctx->desc.order = order;
    return LBM_OK;
}

LBM_API lbm_status lbm_autotune(lbm_ctx *ctx, int32_t retune) {
    CHECK_CTX(ctx);
    if (ctx->desc.mode != LBM_D2Q9) return LBM_OK;  // D3Q27_REF has one launch shape
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    CUDA_TRY(ctx, d2q9_autotune(ctx, retune != 0), "autotune");
    return LBM_OK;
}

LBM_API lbm_status lbm_set_launch(lbm_ctx *ctx, int32_t cells_per_thread, int32_t block_threads, int32_t rows_per_block,
                                  int32_t l2_policy) {
    CHECK_CTX(ctx);
    if (ctx->desc.mode != LBM_D2Q9) return fail(ctx, LBM_ERR_UNSUPPORTED, "lbm_set_launch is D2Q9 only");
    if (!d2q9_shape_valid(ctx, cells_per_thread, block_threads, rows_per_block, l2_policy))
        return fail(ctx, LBM_ERR_INVALID, "launch shape " + std::to_string(cells_per_thread) + "x" +
                                              std::to_string(block_threads) + "x" + std::to_string(rows_per_block) +
                                              " is not valid for this domain and dtype");
    ctx->cells_per_thread = cells_per_thread;
    ctx->block_threads = block_threads;
    ctx->rows_per_block = rows_per_block;
    ctx->l2_policy = l2_policy;
    ctx->tuned = true;
    return LBM_OK;
}

LBM_API lbm_status lbm_set_sweep_alternation(lbm_ctx *ctx, int32_t enabled) {
    CHECK_CTX(ctx);
    ctx->alternate_sweeps = enabled != 0;
    return LBM_OK;
}

LBM_API lbm_status lbm_set_pipeline_wait(lbm_ctx *ctx, int64_t wait_ns, int32_t skip_task) {
    CHECK_CTX(ctx);
    if (wait_ns < 1000 || wait_ns > 10000000000ll)
        return fail(ctx, LBM_ERR_INVALID, "lbm_set_pipeline_wait: wait_ns must be in [1e3, 1e10]");
    if (skip_task < -1) return fail(ctx, LBM_ERR_INVALID, "lbm_set_pipeline_wait: skip_task must be >= -1");
    ctx->pipe_wait_ns = (unsigned long long)wait_ns;
    ctx->pipe_skip_task = skip_task;
    return LBM_OK;
}

LBM_API lbm_status lbm_apply(lbm_ctx *ctx, int32_t op) {
    CHECK_CTX(ctx);
    NvtxRange range("lbm_apply");
    if (ctx->desc.mode != LBM_D3Q27_REF) return fail(ctx, LBM_ERR_UNSUPPORTED, "lbm_apply is D3Q27_REF only");
    if (op != LBM_OP_STREAM && op != LBM_OP_REFLECT && op != LBM_OP_COLLIDE && op != LBM_OP_FLOW)
        return fail(ctx, LBM_ERR_INVALID, "op must be one LBM_OP_* flag");
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    if ((st = d3_prepare(ctx)) != LBM_OK) return st;
    CUDA_TRY(ctx, d3q27_apply(ctx, op), "D3Q27 pass");
    return LBM_OK;
}

LBM_API lbm_status lbm_moments(lbm_ctx *ctx, float *rho, float *ux, float *uy, float *uz) {
    CHECK_CTX(ctx);
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    const size_t n = (size_t)ctx->cells;
    if ((st = ensure_staging(ctx, 4 * n * sizeof(float))) != LBM_OK) return st;
    float *base = static_cast<float *>(ctx->staging);
    float *host[4] = {rho, ux, uy, uz};
    float *dev[4];
    for (int k = 0; k < 4; ++k) dev[k] = host[k] ? base + k * n : nullptr;
    if (ctx->desc.mode == LBM_D2Q9) {
        CUDA_TRY(ctx, d2q9_moments(ctx, dev[0], dev[1], dev[2]), "moments kernel");
        if (uz) std::memset(uz, 0, n * sizeof(float));
        dev[3] = nullptr;
    } else {
        if ((st = d3_prepare(ctx)) != LBM_OK) return st;
        CUDA_TRY(ctx, d3q27_moments(ctx, dev[0], dev[1], dev[2], dev[3]), "moments kernel");
    }
    for (int k = 0; k < 4; ++k)
        if (dev[k])
            CUDA_TRY(ctx, cudaMemcpyAsync(host[k], dev[k], n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
                     "download moments");
    return sync(ctx, "moments");
}

LBM_API lbm_status lbm_conservation(lbm_ctx *ctx, double out[4]) {
    CHECK_CTX(ctx);
    if (!out) return fail(ctx, LBM_ERR_INVALID, "null output");
    lbm_status st = use_device(ctx);
    if (st != LBM_OK) return st;
    double h[4] = {0, 0, 0, 0};
    if (ctx->desc.mode == LBM_D2Q9) {
        CUDA_TRY(ctx, d2q9_conservation(ctx, ctx->result_d), "conservation kernel");
        CUDA_TRY(ctx, cudaMemcpyAsync(h, ctx->result_d, 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "download sums");
    } else {
        if ((st = d3_prepare(ctx)) != LBM_OK) return st;
        CUDA_TRY(ctx, d3q27_conservation(ctx, ctx->result_d), "conservation kernel");
        CUDA_TRY(ctx, cudaMemcpyAsync(h, ctx->result_d, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "download sums");
    }
    if ((st = sync(ctx, "conservation")) != LBM_OK) return st;
    for (int k = 0; k < 4; ++k) out[k] = h[k];
    return LBM_OK;
}

}  // extern "C"
