// Internal declarations shared by the library's translation units (host side).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <string>
#include <vector>

#include "lbm_capi.h"

namespace lbm {

// NVTX range for the duration of a scope (steps, batch rounds, server rounds): visible in Nsight
// Systems / Compute timelines, a no-op without a tool attached
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// D3Q27 directions in the reference's population order (SimCalcFuncs.cu:12, Constants.cpp:6),
// host copy; the inverse of direction q is the q' with c_q' = -c_q (Constants.cpp:7).
constexpr int kD3Q27[27][3] = {
    {0, 0, 0},   {-1, 0, 0},  {0, -1, 0},  {0, 0, -1},  {0, 0, 1},    {0, 1, 0},    {1, 0, 0},
    {-1, -1, 0}, {-1, 0, -1}, {-1, 0, 1},  {-1, 1, 0},  {0, -1, -1},  {0, -1, 1},   {0, 1, -1},
    {0, 1, 1},   {1, -1, 0},  {1, 0, -1},  {1, 0, 1},   {1, 1, 0},    {-1, -1, -1}, {-1, -1, 1},
    {-1, 1, -1}, {-1, 1, 1},  {1, -1, -1}, {1, -1, 1},  {1, 1, -1},   {1, 1, 1}};
constexpr int d3q27_inverse(int q) {
    for (int p = 0; p < 27; ++p)
        if (kD3Q27[p][0] == -kD3Q27[q][0] && kD3Q27[p][1] == -kD3Q27[q][1] && kD3Q27[p][2] == -kD3Q27[q][2])
            return p;
    return -1;
}

// D3Q27_REF gather entry: population `src_pop` of reflecting cell `src_cell` is scattered with
// weight `w` into population `dst_pop` of the target cell (the reference's push of
// SimCalcFuncs.cu:164-186 turned into a pull).  `src_stream` is the cell the reflecting cell's
// population was streamed from (src_cell - c_{src_pop}), or -1 when that lies outside.
struct GatherEntry {
    int32_t src_cell;
    int32_t src_stream;
    float w;
    uint8_t src_pop;
    uint8_t dst_pop;
    uint8_t slot;
    uint8_t pad;
};
static_assert(sizeof(GatherEntry) == 16, "GatherEntry layout");

// D2Q9 per-cell link word: bit j-1 set when population j (1..8) arrives from a wall (half-way
// bounce-back), bit j+7 when that wall moves.  Solid cells hold LINK_SOLID, a pattern no fluid cell
// can have (a moving link always has its bounce bit).
constexpr uint16_t LINK_SOLID = 0x0100;

// struct ReflectionValues of the reference (LatticePoint.h:3-7): 81 slots, direction of slot s in
// bits 5*(s%6) .. 5*(s%6)+4 of dirs[s/6], weight in w[s]
struct ReflRecord {
    int32_t dirs[14];
    float w[81];
};
static_assert(sizeof(ReflRecord) == 380, "ReflectionValues layout");

inline int refl_dir(const ReflRecord &r, int s) {
    return (int)(((uint32_t)r.dirs[s / 6] >> (5 * (s % 6))) & 31u);
}

struct D2Q9Params {
    float omega;        // 1/tau
    float fx, fy;       // body force
    float uwx, uwy;     // moving-wall velocity
    double omega_d, fx_d, fy_d, uwx_d, uwy_d;
};

// device scratch for reductions: per-block partial sums
struct Scratch {
    double *partials = nullptr;
    size_t n = 0;
};

}  // namespace lbm

struct lbm_ctx {
    lbm_desc desc{};
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;

    int64_t cells = 0;
    int64_t pitch = 0;        // D2Q9: elements per row; D3Q27: == cells per plane
    int64_t plane = 0;        // elements per population plane
    int q = 9;
    size_t elem = 4;          // bytes per stored population
    void *f[2] = {nullptr, nullptr};
    int cur = 0;              // f[cur] holds the current state
    uint8_t *flags_d = nullptr;
    uint16_t *links_d = nullptr;
    bool flags_set = false;
    int64_t fluid_cells = 0;
    int64_t steps_done = 0;

    // D3Q27_REF
    int32_t *tgt_cells_d = nullptr;  // target cells of the gather lists
    int32_t *tgt_off_d = nullptr;    // CSR offsets (ntgt + 1)
    lbm::GatherEntry *entries_d = nullptr;
    float *gathered_d = nullptr;     // ntgt x 27: the targets' populations after the gather, before collision
    int32_t *tgt_index_d = nullptr;  // per cell: its index in the target list, or -1
    unsigned *gather_done_d = nullptr;  // blocks of the gather kernel that have written their force partial
    int64_t ntgt = 0, nent = 0;
    float *induced_d = nullptr;      // 27 floats
    bool flow_on = false;
    double *force_acc_d = nullptr;   // running force sum (3 doubles)
    bool force_on = false;

    std::vector<uint8_t> flags_h;    // D3Q27_REF: host copy of the user flag bits
    std::vector<std::pair<int32_t, lbm::ReflRecord>> tables_h;
    bool d3_dirty = true;            // gather lists / device flags need a rebuild
    int eq_mode = LBM_EQ_FLOAT_FLOAT;  // D3Q27_REF: equilibrium evaluation (lbm_set_equilibrium_evaluation)

    lbm::Scratch scratch;
    double *result_d = nullptr;      // small device result buffer (16 doubles)
    void *staging = nullptr;         // host-layout staging buffer, grown on demand
    size_t staging_bytes = 0;

    // D2Q9 step launch shape (set by the autotuner or lbm_set_launch)
    int block_threads = 256;
    int cells_per_thread = 1;
    int rows_per_block = 1;
    int l2_policy = 0;             // vector path: L2 eviction hints (0 none, 1 ld first/st last, 2 ld first)
    unsigned *pipe_status_d = nullptr;  // D2Q9 bulk-copy pipeline: status bits set by a block whose wait gave up
    bool pipe_used = false;             // the pipeline ran since the status was last read
    unsigned long long pipe_wait_ns = 1000000000ull;  // limit of every pipeline wait (lbm_set_pipeline_wait)
    int pipe_skip_task = -1;            // test: task whose copies the producer leaves out (-1: none)
    bool tuned = false;
    bool alternate_sweeps = true;  // visit rows in alternating order on successive steps
    unsigned sweep = 0;

    size_t device_bytes = 0;
};

namespace lbm {

// error helpers
lbm_status fail(lbm_ctx *ctx, lbm_status s, const std::string &msg);
lbm_status cuda_fail(lbm_ctx *ctx, cudaError_t e, const char *what);
lbm_status set_thread_error(lbm_status s, const std::string &msg);

// memory helpers (count device bytes)
lbm_status dalloc(lbm_ctx *ctx, void **p, size_t bytes, const char *what);
void dfree(lbm_ctx *ctx, void *p, size_t bytes);
lbm_status ensure_scratch(lbm_ctx *ctx, size_t n);

// D2Q9 launchers (d2q9.cu)
D2Q9Params d2q9_params(const lbm_desc &d);
cudaError_t d2q9_build_links(lbm_ctx *ctx);
cudaError_t d2q9_init_equilibrium(lbm_ctx *ctx, const float *rho_d, const float *ux_d, const float *uy_d);
cudaError_t d2q9_step(lbm_ctx *ctx, int nsteps);
cudaError_t d2q9_autotune(lbm_ctx *ctx, bool force_retune);
// link words and the fluid-cell count (into count_d) without waiting for them
cudaError_t d2q9_build_links_async(lbm_ctx *ctx, unsigned long long *count_d);
// read and clear the bulk-copy pipeline's status bits (synchronises the context's stream)
unsigned d2q9_take_pipe_status(lbm_ctx *ctx);
bool d2q9_shape_valid(const lbm_ctx *ctx, int v, int tx, int ty, int pol);
cudaError_t d2q9_moments(lbm_ctx *ctx, float *rho_d, float *ux_d, float *uy_d);
cudaError_t d2q9_conservation(lbm_ctx *ctx, double *out_d);
cudaError_t d2q9_load(lbm_ctx *ctx, const void *src_d, int src_dtype, int aos);
cudaError_t d2q9_store(lbm_ctx *ctx, void *dst_d, int dst_dtype, int aos);

// D3Q27_REF launchers (d3q27.cu)
// series_d (optional): the accumulated force after step s is written to series_d[3s..3s+2]
cudaError_t d3q27_step(lbm_ctx *ctx, int nsteps, double *series_d = nullptr);
cudaError_t d3q27_eq_selftest(int64_t n, uint64_t seed, unsigned long long *out_d, cudaStream_t st);
cudaError_t d3q27_division_check(float tau, unsigned long long *bad_d, float *y_d, cudaStream_t st);
cudaError_t d3q27_apply(lbm_ctx *ctx, int op);
cudaError_t d3q27_moments(lbm_ctx *ctx, float *rho_d, float *ux_d, float *uy_d, float *uz_d);
cudaError_t d3q27_conservation(lbm_ctx *ctx, double *out_d);
cudaError_t d3q27_load(lbm_ctx *ctx, const void *src_d, int src_dtype, int aos);
cudaError_t d3q27_store(lbm_ctx *ctx, void *dst_d, int dst_dtype, int aos);

// blocks of the D3Q27_REF gather kernel: one warp per target cell, sixteen per block (d3q27.cu)
inline size_t d3q27_gather_blocks(int64_t ntgt) { return (size_t)((ntgt + 15) / 16); }

// reduction finaliser (common.cu): out[k] (+)= sum_b partials[b*ncomp + k], fixed order
// out[k] (+)= sum over blocks of partials[b][k]; the result is also written to also[k] if given
cudaError_t finalize_sums(cudaStream_t s, const double *partials, int nblocks, int ncomp, double *out,
                          bool accumulate = false, double *also = nullptr);

}  // namespace lbm
