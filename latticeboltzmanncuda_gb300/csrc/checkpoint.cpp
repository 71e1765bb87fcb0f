// Checkpoint and resume of a context (lbm_save / lbm_load / lbm_checkpoint_desc).
//
// The reference has no checkpoint: Lattice::retrieve_data / load_data (Lattice.cpp:73-113) copy the
// AoS records to and from the host, and nothing else of the state (flow source, reflection tables,
// accumulated force, step count) is kept.  A checkpoint here is the context's state as it lies in
// device memory -- the current population buffer in its storage type and layout (structure of
// arrays, row padding included), so a resumed run continues bit for bit -- behind a header with the
// descriptor, and for D3Q27_REF the flag bits, the reflection tables, the flow source, the force
// accumulator and the equilibrium evaluation.  File layout (host byte order):
//   header (struct CkptHeader), flags (cells bytes), tables (n_tables x {int32 cell, 380-byte
//   ReflectionValues record}), populations (q x plane x element bytes)
// The header's checksum covers everything after the header.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "lbm_internal.h"

namespace {

constexpr char kMagic[8] = {'L', 'B', 'M', 'C', 'K', 'P', 'T', '1'};
constexpr uint32_t kVersion = 1;

struct CkptHeader {
    char magic[8];
    uint32_t version;
    uint32_t header_bytes;
    int32_t mode, dtype, nx, ny, nz, periodic;
    float tau, body_force[3], wall_velocity[3];
    int32_t order, force_mode, eq_mode, flow_on, force_on, reserved;
    int64_t steps_done;
    int64_t plane, q, elem;
    int64_t n_tables;
    double force_acc[3];
    float induced[27];
    uint32_t reserved2;
    uint64_t checksum;  // of everything after the header
};
static_assert(sizeof(CkptHeader) % 8 == 0, "header size");

// 64-bit FNV-1a over 8-byte words (tail bytes one by one), continued across calls
struct Hash {
    uint64_t h = 0xcbf29ce484222325ull;
    void add(const void *p, size_t n) {
        const unsigned char *b = static_cast<const unsigned char *>(p);
        size_t i = 0;
        for (; i + 8 <= n; i += 8) {
            uint64_t w;
            std::memcpy(&w, b + i, 8);
            h = (h ^ w) * 0x100000001b3ull;
        }
        for (; i < n; ++i) h = (h ^ b[i]) * 0x100000001b3ull;
    }
};

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

lbm_status read_header(const char *path, CkptHeader &h, File &file, std::string &err) {
    if (!path) {
        err = "null path";
        return LBM_ERR_INVALID;
    }
    file.f = std::fopen(path, "rb");
    if (!file.f) {
        err = std::string("cannot open checkpoint ") + path;
        return LBM_ERR_INVALID;
    }
    if (std::fread(&h, sizeof(h), 1, file.f) != 1 || std::memcmp(h.magic, kMagic, 8) != 0) {
        err = std::string(path) + " is not a checkpoint of this library";
        return LBM_ERR_INVALID;
    }
    if (h.version != kVersion || h.header_bytes != sizeof(CkptHeader)) {
        err = std::string(path) + ": checkpoint version " + std::to_string(h.version) + " is not supported";
        return LBM_ERR_INVALID;
    }
    return LBM_OK;
}

}  // namespace

using namespace lbm;

extern "C" {

LBM_API lbm_status lbm_save(lbm_ctx *ctx, const char *path) {
    if (!ctx) return set_thread_error(LBM_ERR_INVALID, "null context");
    if (!path) return fail(ctx, LBM_ERR_INVALID, "lbm_save: null path");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "lbm_save: synchronise");
    CkptHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.header_bytes = sizeof(CkptHeader);
    const lbm_desc &d = ctx->desc;
    h.mode = d.mode;
    h.dtype = d.dtype;
    h.nx = d.nx;
    h.ny = d.ny;
    h.nz = d.nz;
    h.periodic = d.periodic;
    h.tau = d.tau;
    for (int k = 0; k < 3; ++k) {
        h.body_force[k] = d.body_force[k];
        h.wall_velocity[k] = d.wall_velocity[k];
    }
    h.order = d.order;
    h.force_mode = d.force_mode;
    h.eq_mode = ctx->eq_mode;
    h.flow_on = ctx->flow_on ? 1 : 0;
    h.force_on = ctx->force_on ? 1 : 0;
    h.steps_done = ctx->steps_done;
    h.plane = ctx->plane;
    h.q = ctx->q;
    h.elem = (int64_t)ctx->elem;
    std::vector<uint8_t> flags((size_t)ctx->cells);
    if (d.mode == LBM_D2Q9) {
        e = cudaMemcpy(flags.data(), ctx->flags_d, flags.size(), cudaMemcpyDeviceToHost);
    } else {
        flags = ctx->flags_h;
        h.n_tables = (int64_t)ctx->tables_h.size();
        double acc[4];
        e = cudaMemcpy(acc, ctx->force_acc_d, sizeof(acc), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(h.induced, ctx->induced_d, sizeof(h.induced), cudaMemcpyDeviceToHost);
        for (int k = 0; k < 3; ++k) h.force_acc[k] = acc[k];
    }
    const size_t pop_bytes = (size_t)ctx->plane * ctx->q * ctx->elem;
    std::unique_ptr<unsigned char[]> pops;
    if (e == cudaSuccess) {
        pops.reset(new (std::nothrow) unsigned char[pop_bytes]);
        if (!pops) return fail(ctx, LBM_ERR_OOM, "lbm_save: host buffer for the populations");
        e = cudaMemcpy(pops.get(), ctx->f[ctx->cur], pop_bytes, cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "lbm_save: read the state");
    Hash hs;
    hs.add(flags.data(), flags.size());
    for (const auto &t : ctx->tables_h) {
        hs.add(&t.first, sizeof(int32_t));
        hs.add(&t.second, sizeof(ReflRecord));
    }
    hs.add(pops.get(), pop_bytes);
    h.checksum = hs.h;
    const std::string tmp = std::string(path) + ".tmp";
    bool ok;
    {
        File out;
        out.f = std::fopen(tmp.c_str(), "wb");
        if (!out.f) return fail(ctx, LBM_ERR_INVALID, std::string("lbm_save: cannot write ") + tmp);
        ok = std::fwrite(&h, sizeof(h), 1, out.f) == 1 && std::fwrite(flags.data(), 1, flags.size(), out.f) == flags.size();
        for (const auto &t : ctx->tables_h)
            ok = ok && std::fwrite(&t.first, sizeof(int32_t), 1, out.f) == 1 &&
                 std::fwrite(&t.second, sizeof(ReflRecord), 1, out.f) == 1;
        ok = ok && std::fwrite(pops.get(), 1, pop_bytes, out.f) == pop_bytes;
        ok = ok && std::fflush(out.f) == 0;
    }
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return fail(ctx, LBM_ERR_INVALID, std::string("lbm_save: writing ") + path + " failed");
    }
    return LBM_OK;
}

LBM_API lbm_status lbm_checkpoint_desc(const char *path, lbm_desc *out) {
    if (!out) return set_thread_error(LBM_ERR_INVALID, "lbm_checkpoint_desc: null output");
    CkptHeader h;
    File file;
    std::string err;
    lbm_status st = read_header(path, h, file, err);
    if (st != LBM_OK) return set_thread_error(st, "lbm_checkpoint_desc: " + err);
    lbm_desc_init(out);
    out->mode = h.mode;
    out->dtype = h.dtype;
    out->nx = h.nx;
    out->ny = h.ny;
    out->nz = h.nz;
    out->periodic = h.periodic;
    out->tau = h.tau;
    for (int k = 0; k < 3; ++k) {
        out->body_force[k] = h.body_force[k];
        out->wall_velocity[k] = h.wall_velocity[k];
    }
    out->order = h.order;
    out->force_mode = h.force_mode;
    return LBM_OK;
}

LBM_API lbm_status lbm_load(lbm_ctx *ctx, const char *path) {
    if (!ctx) return set_thread_error(LBM_ERR_INVALID, "null context");
    CkptHeader h;
    File file;
    std::string err;
    lbm_status st = read_header(path, h, file, err);
    if (st != LBM_OK) return fail(ctx, st, "lbm_load: " + err);
    const lbm_desc &d = ctx->desc;
    if (h.mode != d.mode || h.dtype != d.dtype || h.nx != d.nx || h.ny != d.ny || h.nz != d.nz ||
        h.plane != ctx->plane || h.q != ctx->q || h.elem != (int64_t)ctx->elem)
        return fail(ctx, LBM_ERR_INVALID,
                    "lbm_load: the checkpoint's mode, storage type or size differ from the context's "
                    "(lbm_checkpoint_desc gives a descriptor to create a matching context)");
    if (h.n_tables < 0 || h.n_tables > ctx->cells || (d.mode == LBM_D2Q9 && h.n_tables != 0))
        return fail(ctx, LBM_ERR_INVALID, "lbm_load: corrupt checkpoint (table count)");
    std::vector<uint8_t> flags((size_t)ctx->cells);
    std::vector<int32_t> cells((size_t)h.n_tables);
    std::vector<ReflRecord> recs((size_t)h.n_tables);
    const size_t pop_bytes = (size_t)ctx->plane * ctx->q * ctx->elem;
    std::unique_ptr<unsigned char[]> pops(new (std::nothrow) unsigned char[pop_bytes]);
    if (!pops) return fail(ctx, LBM_ERR_OOM, "lbm_load: host buffer for the populations");
    Hash hs;
    bool ok = std::fread(flags.data(), 1, flags.size(), file.f) == flags.size();
    hs.add(flags.data(), flags.size());
    for (int64_t i = 0; ok && i < h.n_tables; ++i) {
        ok = std::fread(&cells[(size_t)i], sizeof(int32_t), 1, file.f) == 1 &&
             std::fread(&recs[(size_t)i], sizeof(ReflRecord), 1, file.f) == 1;
        hs.add(&cells[(size_t)i], sizeof(int32_t));
        hs.add(&recs[(size_t)i], sizeof(ReflRecord));
    }
    ok = ok && std::fread(pops.get(), 1, pop_bytes, file.f) == pop_bytes;
    if (ok) hs.add(pops.get(), pop_bytes);
    if (!ok) return fail(ctx, LBM_ERR_INVALID, std::string("lbm_load: ") + path + " is truncated");
    if (hs.h != h.checksum) return fail(ctx, LBM_ERR_INVALID, std::string("lbm_load: checksum mismatch in ") + path);

    // descriptor parameters of the checkpoint, then the geometry, then the state
    ctx->desc.periodic = h.periodic;
    ctx->desc.order = h.order;
    ctx->desc.force_mode = h.force_mode;
    if ((st = lbm_set_params(ctx, h.tau, h.body_force, h.wall_velocity)) != LBM_OK) return st;
    if (d.mode == LBM_D3Q27_REF) {
        if ((st = lbm_set_reflection_tables(ctx, h.n_tables, cells.data(), recs.data())) != LBM_OK) return st;
        if ((st = lbm_set_equilibrium_evaluation(ctx, h.eq_mode)) != LBM_OK) return st;
    }
    if ((st = lbm_set_flags(ctx, flags.data())) != LBM_OK) return st;
    if (d.mode == LBM_D3Q27_REF) {
        if ((st = lbm_set_flow(ctx, nullptr, h.flow_on ? h.induced : nullptr)) != LBM_OK) return st;
        const float acc[3] = {(float)h.force_acc[0], (float)h.force_acc[1], (float)h.force_acc[2]};
        if ((st = lbm_set_force(ctx, acc, h.force_on)) != LBM_OK) return st;
        // the running sum in full FP64, not rounded through the float interface
        const double full[4] = {h.force_acc[0], h.force_acc[1], h.force_acc[2], 0.0};
        const cudaError_t e = cudaMemcpy(ctx->force_acc_d, full, sizeof(full), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "lbm_load: force");
    }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpy(ctx->f[ctx->cur], pops.get(), pop_bytes, cudaMemcpyHostToDevice);
    // into the other buffer as well: the D2Q9 step never writes solid cells, so both buffers must
    // agree there (its fluid cells are overwritten by the next step)
    if (e == cudaSuccess && ctx->f[ctx->cur ^ 1])
        e = cudaMemcpy(ctx->f[ctx->cur ^ 1], pops.get(), pop_bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "lbm_load: populations");
    ctx->steps_done = h.steps_done;
    return LBM_OK;
}

}  // extern "C"
