// Batched D2Q9: many independent domains of uneven size, tau, forcing and obstacle mask advance
// together, one kernel launch per time step for all of them, each launch the programmatic dependent
// of the one before (lbm_batch_set_persistent: one persistent cooperative launch per step sequence
// instead, its blocks meeting after each step).
//
// Each domain (a "slot") owns one allocation -- its two population buffers, link words, flags and
// fluid-cell count -- made when it is added, so slots come and go without moving anyone else's
// state (the serving loop admits and retires requests between rounds).  Every block of a launch
// updates one tile of one slot with the same vectorised update as the single-domain kernel, so a
// domain's populations are bit-identical whether it runs alone or in any mix.  Tiles are ordered
// slot by slot, rows ascending; odd steps walk them backwards (each step starts where the previous
// one ended, on data still in L2).  Up to PARAM_SLOTS live slots (FP32, 16-bit storage) the slot
// descriptors (size, buffer base, parity, step budget, relaxation rate, force, wall velocity,
// periodicity) and the first tile of every slot travel in the kernel's parameter block, a block
// finds its slot by a binary search over those; with 16-bit storage a tile is a run of TX * TY * V
// consecutive cells of the slot's padded cell array (and its first thread prefetches into L2 the
// tile 32k cells further along the slot), with FP32 a band of TY rows of TX * V cells; beyond that,
// and for FP64, a device table of descriptors and a tile list (slot, x-chunk, first row: TY rows x
// TX * V cells) do.  The tile shape (V, TX, TY) is picked by the autotuner from timings on the batch
// itself.
//
// Nothing on the serving path waits for the device: adding a slot (flags upload, link words,
// fluid-cell count, equilibrium), the table uploads before a launch sequence, freeing a slot and
// reading a slot's moments back through a ticket (lbm_batch_moments_async) are all queued on the
// batch stream, with host data staged through pinned blocks that are reused once the copy that
// last used them has completed.  The host can thus prepare the next round of a request loop
// while the device runs the current one.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "d2q9_vec.cuh"
#include "lbm_internal.h"
#include "pdl.cuh"

namespace lbm {
lbm_status set_thread_error(lbm_status s, const std::string &msg);
}

using namespace lbm;

namespace {

struct SlotDesc {  // device descriptor, one per slot
    void *f[2];
    const uint16_t *links;
    int nx, ny, pitch, plane;
    int periodic, force;
    int cur;   // buffer holding the current state at the start of the launch sequence
    int stop;  // steps this slot takes in the launch sequence (its remaining step budget)
    D2Q9Params prm;
};

struct Tile {
    int slot, xchunk, y0, pad;
};

// A pinned host block for asynchronous copies; reusable once `done` (recorded after the last copy
// that used it) has completed.
struct PinnedBlock {
    void *p = nullptr;
    size_t bytes = 0;
    cudaEvent_t done = nullptr;
};

// An asynchronous read-back of a slot's moments: 3 n floats in a pinned block, ready at `done`.
struct Pending {
    size_t block;
    size_t n;
    cudaEvent_t done;
};

struct Slot {
    bool live = false;
    lbm_desc desc{};
    int pitch = 0;
    int64_t plane = 0;
    void *f[2] = {nullptr, nullptr};
    uint16_t *links = nullptr;
    uint8_t *flags = nullptr;
    unsigned long long *count_d = nullptr;  // fluid-cell count, behind the flags in their allocation
    int cur = 0;
    int64_t steps_done = 0;
    int64_t limit = -1;  // steps the slot may still take (-1: no limit)
    int64_t fluid = -1;  // -1 until the device count has been read
    size_t bytes = 0;
};

// bytes of a slot's flag allocation: the flags, padded to 8 bytes, then the fluid-cell count
size_t flags_bytes(int nx, int ny) { return ((size_t)nx * ny + 7) / 8 * 8 + 8; }

// Table path: one block per tile.  The tile's slot descriptor is copied into registers, so no field
// is re-read from global memory after the population stores.  (A persistent grid-stride loop over
// the tiles measured slower: it keeps ~40 more registers live and halves the occupancy.)
template <class S, int V>
__device__ __forceinline__ void batch_tile(const SlotDesc *__restrict__ slots, const Tile *__restrict__ tiles,
                                           int ntiles, int step, int reverse) {
    const int t = reverse ? ntiles - 1 - (int)blockIdx.x : (int)blockIdx.x;
    const Tile tile = tiles[t];
    const SlotDesc D = slots[tile.slot];
    if (step >= D.stop) return;  // the slot has used its step budget (uniform per block)
    const int y = tile.y0 + (int)threadIdx.y;
    if (y >= D.ny) return;  // uniform per warp
    const int x0 = (tile.xchunk * (int)blockDim.x + (int)threadIdx.x) * V;
    const int cur = (D.cur + step) & 1;
    const S *src = static_cast<const S *>(D.f[cur]);
    S *dst = static_cast<S *>(D.f[cur ^ 1]);
    if (D.force)
        d2q9::step_vec<S, V, true, int>(src, dst, D.links, x0, y, D.nx, D.ny, D.pitch, D.plane, D.periodic, D.prm);
    else
        d2q9::step_vec<S, V, false, int>(src, dst, D.links, x0, y, D.nx, D.ny, D.pitch, D.plane, D.periodic, D.prm);
}

template <class S, int V>
__global__ void __launch_bounds__(256) batch_step_kernel(const SlotDesc *__restrict__ slots,
                                                         const Tile *__restrict__ tiles, int ntiles, int step,
                                                         int reverse) {
    wait_prerequisite_grids();  // a programmatic dependent of the launch before (launch_v)
    allow_dependent_launch();
    batch_tile<S, V>(slots, tiles, ntiles, step, reverse);
}

// 16-bit storage, 4-wide vectors: registers held to 64 so that 32 warps fit per SM (measured 5 %
// faster on the mixed serve domains; FP32 measured slower with the same bound and keeps the kernel
// above)
template <class S, int V>
__global__ void __launch_bounds__(256, 4) batch_step_kernel_occ(const SlotDesc *__restrict__ slots,
                                                                const Tile *__restrict__ tiles, int ntiles, int step,
                                                                int reverse) {
    wait_prerequisite_grids();  // a programmatic dependent of the launch before (launch_v)
    allow_dependent_launch();
    batch_tile<S, V>(slots, tiles, ntiles, step, reverse);
}

// Batches of up to PARAM_SLOTS live slots (FP32 and 16-bit storage) pass their descriptors and the
// first tile of every slot in the kernel's parameter block (constant memory, served to all blocks
// of an SM by the constant cache): a block finds its slot by a binary search over the tile offsets
// and derives its row band and column chunk, with no dependent global load before its own
// population loads.  Larger batches (and FP64) read the descriptor and tile tables from global
// memory as above.
constexpr int PARAM_SLOTS = 540;

struct SlotDescP {  // 56 bytes; pitch, plane, buffers and link words follow from these
    void *base;  // the slot's allocation: buffer A, buffer B (9 planes each), link words
    int nx, ny;
    int bits;    // periodic (bits 0-1), force (bit 2), current buffer at the sequence start (bit 3),
                 // shift of the division by the pitch (bits 8-12)
    int stop;    // steps this slot takes in the launch sequence
    unsigned magic;  // flat tiles: multiplier of the division by the pitch (Granlund-Montgomery)
    int chunks;      // row-band tiles: column chunks per row band
    float omega, fx, fy, uwx, uwy;
};

struct BatchParams {
    int n;       // slots in the block
    int ntiles;  // tiles of the launch
    int start[PARAM_SLOTS];
    SlotDescP d[PARAM_SLOTS];
};

static_assert(sizeof(BatchParams) <= 32764, "kernel parameter block limit");

// Parameter-block tiles.  16-bit storage: flat -- tile j of a slot is the run of blockDim.x *
// blockDim.y * V consecutive cells starting at j * blockDim.x * blockDim.y * V of the slot's padded
// cell array [0, pitch * ny), row after row (step_vec_flat), so a row costs at most its 31 padding
// cells of idle lanes instead of the rest of a column chunk, and only a slot's last tile is ragged.
// FP32: row bands -- tile j is the column chunk j % chunks of the band of blockDim.y rows j / chunks,
// each warp one row (step_vec).  Measured on the 512-domain batch: FP16 104.0k against 102.3k MLUPS
// with row bands, FP32 81.8k against 85.6k with flat tiles.  Either way a block finds its slot by a
// binary search over the slots' first tiles in the parameter block: the loop and its loads are
// uniform, so the descriptor fields come from the constant bank.  (An 8-byte tile record per block
// read from global memory instead measured 1-4 % slower with the flat tiles.)
template <class S>
constexpr bool flat_tiles() {
    return sizeof(S) == 2;
}

// L2 prefetch of the flat tiles that start soon: the block's first thread asks L2 for the ten
// segments (nine planes, with the row shift of their pull, and the link words) of the tile
// PREFETCH_CELLS cells further along its slot in the sweep's direction (`cp.async.bulk.prefetch`,
// no registers held and nothing to wait for), so those tiles' loads find their lines in L2.
// Measured on the 512-domain batch and the serve mix (FP16): 118.0k -> 124.7k and 127.6k ->
// 136.4k MLUPS; 8k to 64k cells ahead all within 2 %; on the single-domain kernel the same
// prefetch measured slower.
constexpr int PREFETCH_CELLS = 32768;

__device__ __forceinline__ void prefetch_l2(const void *ptr, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(ptr), "r"(bytes) : "memory");
}

// Tile t of the launch sequence's step `step` (POL 3: the loads at L2, coherent with the stores of
// the previous step in the same launch); dir +1 / -1: the sweep's direction for the L2 prefetch of
// flat tiles (0: none).
template <class S, int V, int POL = 0>
__device__ __forceinline__ void batch_tile_p(const BatchParams &p, int t, int step, int dir = 0) {
    int lo = 0, hi = p.n - 1;
    while (lo < hi) {  // the last slot whose first tile is at or before t (uniform per block)
        const int mid = (lo + hi + 1) >> 1;
        if (p.start[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const int slot = lo, tile = t - p.start[lo];
    const SlotDescP &D = p.d[slot];
    if (step >= D.stop) return;  // the slot has used its step budget
    const int pitch = (D.nx + 31) & ~31, plane = pitch * D.ny;
    int x0, y;
    bool active = true;
    if constexpr (flat_tiles<S>()) {
        const int k = (int)threadIdx.y * (int)blockDim.x + (int)threadIdx.x;
        const int first = tile * (int)(blockDim.x * blockDim.y) * V;
        if (first + (k & ~31) * V >= plane) return;  // the warp lies past the slot's last cell (uniform)
        int i = first + k * V;
        active = i < plane;
        if (!active) i = plane - V;  // in bounds; shuffles only, no store
        // i / pitch by multiply-high (pitch >= 32, so the pre-shift is 1)
        const uint32_t th = __umulhi(D.magic, (uint32_t)i);
        y = (int)((th + (((uint32_t)i - th) >> 1)) >> ((D.bits >> 8) & 31));
        x0 = i - y * pitch;
    } else {
        const int band = tile / D.chunks, xchunk = tile - band * D.chunks;
        y = band * (int)blockDim.y + (int)threadIdx.y;
        if (y >= D.ny) return;  // uniform per warp
        x0 = (xchunk * (int)blockDim.x + (int)threadIdx.x) * V;
    }
    const int cur = ((D.bits >> 3) + step) & 1;
    S *const a = static_cast<S *>(D.base);
    const S *src = a + (size_t)cur * 9 * plane;
    S *dst = a + (size_t)(cur ^ 1) * 9 * plane;
    const uint16_t *links = reinterpret_cast<const uint16_t *>(a + (size_t)18 * plane);
    if constexpr (flat_tiles<S>()) {
        if (dir != 0 && threadIdx.x == 0 && threadIdx.y == 0) {
            // segments of per cells, every offset a multiple of 32 cells (16-byte aligned) and
            // clamped into the slot's planes
            const int per = (int)(blockDim.x * blockDim.y) * V;
            const int tf = tile + dir * (PREFETCH_CELLS / per);
            if (plane >= per && tf >= 0 && (int64_t)tf * per < (int64_t)plane) {
                const int first = min(tf * per, plane - per);
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    const int dy = d2q9::cy(q);  // the pull of population q reads row y - c_y(q)
                    const int o = max(0, min(first - dy * pitch, plane - per));
                    prefetch_l2(src + (size_t)q * plane + o, (unsigned)(per * sizeof(S)));
                }
                prefetch_l2(links + first, (unsigned)(per * sizeof(uint16_t)));
            }
        }
    }
    D2Q9Params prm;
    prm.omega = D.omega;
    prm.fx = D.fx;
    prm.fy = D.fy;
    prm.uwx = D.uwx;
    prm.uwy = D.uwy;
    prm.omega_d = prm.fx_d = prm.fy_d = prm.uwx_d = prm.uwy_d = 0.0;  // FP64 storage uses the table path
    const int periodic = D.bits & 3;
    if constexpr (flat_tiles<S>()) {
        if (D.bits & 4)
            d2q9::step_vec_flat<S, V, true, int, POL>(src, dst, links, x0, y, D.nx, D.ny, pitch, plane, periodic, prm,
                                                      active);
        else
            d2q9::step_vec_flat<S, V, false, int, POL>(src, dst, links, x0, y, D.nx, D.ny, pitch, plane, periodic, prm,
                                                       active);
    } else {
        if (D.bits & 4)
            d2q9::step_vec<S, V, true, int, POL>(src, dst, links, x0, y, D.nx, D.ny, pitch, plane, periodic, prm);
        else
            d2q9::step_vec<S, V, false, int, POL>(src, dst, links, x0, y, D.nx, D.ny, pitch, plane, periodic, prm);
    }
}

// registers held to 64 for 2- and 4-wide vectors (32 warps per SM) and 128 for 8-wide ones: the
// descriptor fields read from the parameter block otherwise stay in registers and cost occupancy.
// (FP32 4-wide at 64 registers, a few bytes spilled, measured 90.2k MLUPS on the 512-domain batch
// against 87.3k at 85.)
__host__ __device__ constexpr int batch_min_blocks(int v) { return v == 8 ? 2 : 4; }

__device__ __forceinline__ int launch_tile(int ntiles, int reverse) {
    return reverse ? ntiles - 1 - (int)blockIdx.x : (int)blockIdx.x;
}

template <class S, int V>
__global__ void __launch_bounds__(256, batch_min_blocks(V)) batch_step_kernel_p(const __grid_constant__ BatchParams p,
                                                                               int step, int reverse) {
    wait_prerequisite_grids();  // a programmatic dependent of the launch before (launch_v)
    allow_dependent_launch();
    batch_tile_p<S, V>(p, launch_tile(p.ntiles, reverse), step, reverse ? -1 : 1);
}

template <class S, int V>
__global__ void __launch_bounds__(256, 4) batch_step_kernel_p_occ(const __grid_constant__ BatchParams p, int step,
                                                                  int reverse) {
    wait_prerequisite_grids();  // a programmatic dependent of the launch before (launch_v)
    allow_dependent_launch();
    batch_tile_p<S, V>(p, launch_tile(p.ntiles, reverse), step, reverse ? -1 : 1);
}

// Persistent launch: one cooperative launch runs a whole step sequence.  Its blocks (no more than
// fit on the GPU at once) take the step's tiles b, b + gridDim.x, ... and then meet all other
// blocks before the next step, whose loads go to L2 (the previous step's stores of other SMs are
// there, while this SM's L1 may hold lines of the buffer from two steps ago).  For batches of few
// cells, where one launch per step costs more than the step itself.
struct GridSync {
    unsigned int arrived;  // block arrivals since the launch began
    unsigned int status;   // nonzero: a block gave up waiting for the others
};

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Every block of the launch arrives; the first thread of each then waits until `target` arrivals
// are counted, at most limit_ns (then it records the failure in g->status, and every block that
// sees it ends its launch).  `skip`: the block does not arrive (a diagnostic of the wait limit).
// Returns false when the sequence must stop.
__device__ bool grid_meet(GridSync *g, unsigned target, int64_t limit_ns, bool skip) {
    __shared__ int ok;  // the first thread's verdict, the same for the whole block
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();  // this block's stores before its arrival
        if (!skip) atomicAdd(&g->arrived, 1u);
        const uint64_t t0 = global_ns();
        volatile unsigned *arrived = &g->arrived, *status = &g->status;
        while (*arrived < target && *status == 0) {
            if ((int64_t)(global_ns() - t0) > limit_ns) {
                atomicOr(&g->status, 1u);
                break;
            }
            __nanosleep(64);
        }
        __threadfence();  // the other blocks' stores before this block's next loads
        ok = *status == 0;
    }
    __syncthreads();
    return ok != 0;
}

// registers held to 128 (the step-loop state comes on top of the tile's; a batch that runs
// persistent is small, so occupancy counts less than spills)
template <class S>
constexpr int persist_min_blocks() {
    return 2;
}

template <class S>
__global__ void __launch_bounds__(256, persist_min_blocks<S>())
    batch_persistent_kernel(const __grid_constant__ BatchParams p, int nsteps, int sweep0, GridSync *g,
                            int64_t limit_ns, int skip_block) {
    for (int s = 0; s < nsteps; ++s) {
        const int reverse = (sweep0 + s) & 1;
        for (int b = (int)blockIdx.x; b < p.ntiles; b += (int)gridDim.x)
            batch_tile_p<S, 4, 3>(p, reverse ? p.ntiles - 1 - b : b, s);
        if (s + 1 < nsteps &&
            !grid_meet(g, (unsigned)(s + 1) * gridDim.x, limit_ns, s == 0 && (int)blockIdx.x == skip_block))
            return;
    }
}

size_t dsize(int dtype) { return dtype == LBM_F64 ? 8 : (dtype == LBM_F32 ? 4 : 2); }

template <class S>
constexpr bool vec_ok(int v) {
    return (sizeof(S) == 4 && (v == 2 || v == 4)) || (sizeof(S) == 2 && (v == 2 || v == 4 || v == 8)) ||
           (sizeof(S) == 8 && v == 2);
}

}  // namespace

struct lbm_batch {
    int dtype = LBM_F32;
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    std::vector<Slot> slots;
    // device tables (rebuilt when the live set or the shape changes)
    SlotDesc *desc_d = nullptr;
    size_t desc_cap = 0;
    Tile *tiles_d = nullptr;
    size_t tiles_cap = 0;
    int ntiles = 0;
    bool dirty = true;        // descriptors need rewriting
    bool tiles_dirty = true;  // the live set or the tile shape changed: the tile list too
    // tile shape
    int v = 4, tx = 32, ty = 4;
    bool tuned = false;
    bool fixed = false;      // shape set by lbm_batch_set_launch: never tuned
    int64_t live_cells = 0;  // cells of the live slots
    int64_t tuned_cells = 0; // live cells when the shape was last tuned
    int32_t tunings = 0;
    unsigned sweep = 0;
    int64_t device_bytes = 0;
    // persistent staging for slot I/O and a small result buffer (no allocation per call)
    void *staging = nullptr;
    size_t staging_bytes = 0;
    double *result_d = nullptr;
    std::vector<PinnedBlock> pinned;
    std::map<int64_t, Pending> pending;  // read-backs by ticket
    bool use_params = false;             // the launch takes the descriptors in its parameter block
    BatchParams params{};
    int64_t next_ticket = 1;
    // persistent launches: mode (0 never, the default: one launch per step, each the programmatic
    // dependent of the one before, measured faster at every batch size; 1 batches of at most
    // PERSIST_CELLS live cells; 2 whenever the launch allows it), the limit of their waits, a block
    // that does not arrive (diagnostic)
    int persist = 0;
    int64_t persist_wait_ns = 1000000000;
    int persist_skip = -1;
    GridSync *sync_d = nullptr;
    bool sync_d_init = false;
    int persist_launches = 0;  // persistent launches so far (lbm_batch_info)
};

namespace {

lbm_status bfail(lbm_batch *b, lbm_status s, const std::string &m) {
    if (b) b->err = m;
    return lbm::set_thread_error(s, m);
}

#define BCUDA(b, call, what)                                                                                  \
    do {                                                                                                      \
        cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess)                                                                                \
            return bfail(b, e_ == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA,                     \
                         std::string(what) + ": " + cudaGetErrorString(e_));                                  \
    } while (0)

// below this many live cells the batch runs the default shape and does not tune
constexpr int64_t TUNE_CELLS = (int64_t)1 << 24;

// default tile shape (the autotuner's choice on the mixed serve domains: 16-bit 4 x 32 x 4,
// FP32 4 x 32 x 2)
void default_shape(int dtype, int &v, int &tx, int &ty) {
    v = dtype == LBM_F64 ? 2 : 4;
    tx = 32;
    ty = dtype == LBM_F32 ? 2 : 4;
}

bool shape_ok(int dtype, int v, int tx, int ty) {
    if (tx < 32 || tx % 32 || ty < 1 || tx * ty > 256) return false;
    switch (dtype) {
        case LBM_F32: return vec_ok<float>(v);
        case LBM_F16S: return vec_ok<__half>(v);
        case LBM_BF16S: return vec_ok<__nv_bfloat16>(v);
        case LBM_F64: return vec_ok<double>(v);
    }
    return false;
}

// Slot set-up and I/O run the single-domain kernels on a temporary lbm_ctx that views the slot's
// buffers (the view owns nothing).
struct CtxView {
    lbm_ctx c;
    CtxView(lbm_batch *b, Slot &s) {
        c.desc = s.desc;
        c.desc.dtype = b->dtype;
        c.device = b->device;
        c.stream = b->stream;
        c.cells = (int64_t)s.desc.nx * s.desc.ny;
        c.pitch = s.pitch;
        c.plane = s.plane;
        c.q = 9;
        c.elem = dsize(b->dtype);
        c.f[0] = s.f[0];
        c.f[1] = s.f[1];
        c.cur = s.cur;
        c.flags_d = s.flags;
        c.links_d = s.links;
        c.flags_set = true;
        c.result_d = nullptr;
    }
    ~CtxView() {
        // the view owns nothing
        c.f[0] = c.f[1] = nullptr;
        c.flags_d = nullptr;
        c.links_d = nullptr;
        c.staging = nullptr;
        c.result_d = nullptr;
        c.scratch.partials = nullptr;
    }
};

// Slot buffers come from the device's stream-ordered memory pool on the batch stream: freeing a
// slot does not synchronise the device (its memory returns to the pool once the work queued before
// the free has run), and a later slot reuses the pooled memory without a new device allocation.
void free_slot(lbm_batch *b, Slot &s) {
    if (s.f[0]) cudaFreeAsync(s.f[0], b->stream);  // the slot's one allocation (see slot_layout)
    s.f[0] = s.f[1] = nullptr;
    s.links = nullptr;
    s.flags = nullptr;
}

bool block_in_use(const lbm_batch *b, size_t k) {
    for (const auto &kv : b->pending)
        if (kv.second.block == k) return true;
    return false;
}

// A free pinned block of at least n bytes (the smallest that fits; a new one when none is free).
// Sets *index; the caller records the block's event after queuing the copy that uses it.
lbm_status pinned_get(lbm_batch *b, size_t n, size_t *index) {
    size_t best = SIZE_MAX;
    for (size_t k = 0; k < b->pinned.size(); ++k) {
        const PinnedBlock &pb = b->pinned[k];
        if (pb.bytes < n || (best != SIZE_MAX && pb.bytes >= b->pinned[best].bytes)) continue;
        if (cudaEventQuery(pb.done) != cudaSuccess || block_in_use(b, k)) continue;
        best = k;
    }
    cudaGetLastError();  // cudaEventQuery reports cudaErrorNotReady for blocks still in use
    if (best == SIZE_MAX) {
        PinnedBlock pb;
        pb.bytes = std::max<size_t>(n, (size_t)1 << 20);
        BCUDA(b, cudaHostAlloc(&pb.p, pb.bytes, cudaHostAllocDefault), "batch: pinned staging");
        if (cudaEventCreateWithFlags(&pb.done, cudaEventDisableTiming) != cudaSuccess) {
            cudaFreeHost(pb.p);
            return bfail(b, LBM_ERR_CUDA, "batch: pinned staging event");
        }
        b->pinned.push_back(pb);
        best = b->pinned.size() - 1;
    }
    *index = best;
    return LBM_OK;
}

// Copy n host bytes to device memory without waiting: through a pinned block, on the batch stream.
lbm_status upload_async(lbm_batch *b, void *dst_d, const void *src_h, size_t n, const char *what) {
    if (n == 0) return LBM_OK;
    size_t k;
    lbm_status st = pinned_get(b, n, &k);
    if (st != LBM_OK) return st;
    std::memcpy(b->pinned[k].p, src_h, n);
    BCUDA(b, cudaMemcpyAsync(dst_d, b->pinned[k].p, n, cudaMemcpyHostToDevice, b->stream), what);
    BCUDA(b, cudaEventRecord(b->pinned[k].done, b->stream), what);
    return LBM_OK;
}

// Grow a device table to hold n elements of `size` bytes, stream-ordered (launches queued before
// keep the old table until they have run).
lbm_status grow_table(lbm_batch *b, void **table, size_t *cap, size_t n, size_t size, size_t min_cap, const char *what) {
    if (n <= *cap) return LBM_OK;
    if (*table) cudaFreeAsync(*table, b->stream);
    *table = nullptr;
    *cap = 0;
    const size_t want = std::max(n + n / 4, min_cap);
    BCUDA(b, cudaMallocAsync(table, want * size, b->stream), what);
    *cap = want;
    return LBM_OK;
}

// steps slot s takes in a launch sequence of nsteps
int64_t advance_of(const Slot &s, int64_t nsteps) { return s.limit < 0 ? nsteps : std::min(nsteps, s.limit); }

// Descriptors and tiles for a launch sequence of nsteps.  The tile list changes only with the live
// set or the shape (b->tiles_dirty); the descriptors carry each slot's stop step (slots with a step
// budget stop early) and are rewritten for every launch sequence while some slot has a budget.
// Tiles of a slot whose budget is used up stay in the list: their blocks return at once.
lbm_status rebuild(lbm_batch *b, int64_t nsteps) {
    bool limited = false;
    int live = 0;
    for (const Slot &s : b->slots) {
        limited |= s.live && s.limit >= 0;
        live += s.live ? 1 : 0;
    }
    if (!b->dirty && !b->tiles_dirty && !limited) return LBM_OK;
    // the parameter-block path: FP32 / 16-bit storage and at most PARAM_SLOTS slots
    const bool params_ok = b->dtype != LBM_F64 && live <= PARAM_SLOTS;
    if (params_ok) {  // descriptors as kernel parameters
        BatchParams &p = b->params;
        p.n = 0;
        int ntiles = 0;
        for (const Slot &s : b->slots) {
            if (!s.live) continue;
            SlotDescP &d = p.d[p.n];
            const int64_t adv = advance_of(s, nsteps);
            d.stop = s.limit < 0 ? INT32_MAX : (int)std::min<int64_t>(adv, INT32_MAX);
            d.base = s.f[0];
            d.nx = s.desc.nx;
            d.ny = s.desc.ny;
            const bool force = s.desc.body_force[0] != 0.0f || s.desc.body_force[1] != 0.0f;
            // division by the pitch (>= 32): multiplier m and shift l - 1, l = ceil(log2 pitch)
            int l = 0;
            while ((1ll << l) < s.pitch) ++l;
            d.magic = (unsigned)((((uint64_t)1 << 32) * (((uint64_t)1 << l) - (uint64_t)s.pitch)) / (uint64_t)s.pitch + 1);
            d.bits = (s.desc.periodic & 3) | (force ? 4 : 0) | (s.cur ? 8 : 0) | ((l - 1) << 8);
            const int per_tile = b->tx * b->ty * b->v;
            d.chunks = (s.pitch / b->v + b->tx - 1) / b->tx;
            const int ntile_slot = dsize(b->dtype) == 2 ? (int)((s.plane + per_tile - 1) / per_tile)
                                                        : d.chunks * ((s.desc.ny + b->ty - 1) / b->ty);
            const D2Q9Params prm = d2q9_params(s.desc);
            d.omega = prm.omega;
            d.fx = prm.fx;
            d.fy = prm.fy;
            d.uwx = prm.uwx;
            d.uwy = prm.uwy;
            p.start[p.n] = ntiles;
            ntiles += ntile_slot;
            ++p.n;
        }
        p.ntiles = ntiles;
        b->ntiles = ntiles;
        b->use_params = true;
        b->dirty = false;
        b->tiles_dirty = false;
        return LBM_OK;
    }
    std::vector<SlotDesc> descs(b->slots.size());
    std::vector<Tile> tiles;
    const bool retile = b->tiles_dirty || b->use_params;  // the tile table is stale after parameter launches
    b->use_params = false;
    for (size_t i = 0; i < b->slots.size(); ++i) {
        const Slot &s = b->slots[i];
        SlotDesc &d = descs[i];
        std::memset(&d, 0, sizeof(d));
        if (!s.live) continue;
        const int64_t adv = advance_of(s, nsteps);
        // only slots with a step budget stop early; their tables are rebuilt for every launch sequence
        d.stop = s.limit < 0 ? INT32_MAX : (int)std::min<int64_t>(adv, INT32_MAX);
        d.f[0] = s.f[0];
        d.f[1] = s.f[1];
        d.links = s.links;
        d.nx = s.desc.nx;
        d.ny = s.desc.ny;
        d.pitch = s.pitch;
        d.plane = (int)s.plane;
        d.periodic = s.desc.periodic;
        d.force = (s.desc.body_force[0] != 0.0f || s.desc.body_force[1] != 0.0f) ? 1 : 0;
        d.cur = s.cur;
        d.prm = d2q9_params(s.desc);
        if (!retile) continue;
        const int chunks = (s.pitch / b->v + b->tx - 1) / b->tx;
        for (int y0 = 0; y0 < s.desc.ny; y0 += b->ty)
            for (int xc = 0; xc < chunks; ++xc) tiles.push_back(Tile{(int)i, xc, y0, 0});
    }
    // uploads queued behind the launches that still read the old tables
    lbm_status st = grow_table(b, (void **)&b->desc_d, &b->desc_cap, descs.size(), sizeof(SlotDesc), 64,
                               "batch: descriptor table");
    if (st == LBM_OK)
        st = upload_async(b, b->desc_d, descs.data(), descs.size() * sizeof(SlotDesc), "batch: upload descriptors");
    if (st != LBM_OK) return st;
    if (retile) {
        st = grow_table(b, (void **)&b->tiles_d, &b->tiles_cap, tiles.size(), sizeof(Tile), 1024, "batch: tile table");
        if (st == LBM_OK) st = upload_async(b, b->tiles_d, tiles.data(), tiles.size() * sizeof(Tile), "batch: upload tiles");
        if (st != LBM_OK) return st;
        b->ntiles = (int)tiles.size();
    }
    b->dirty = false;
    b->tiles_dirty = false;
    return LBM_OK;
}

template <class S, int V>
cudaError_t launch_v(lbm_batch *b, int step, int reverse) {
    // every step kernel is the programmatic dependent of the launch before it: its blocks wait for
    // that grid at entry and may be scheduled while its last blocks finish
    const dim3 block(b->tx, b->ty);
    const dim3 grid((unsigned)b->ntiles);
    cudaError_t e = cudaErrorInvalidValue;
    if (b->use_params) {
        if constexpr (sizeof(S) == 2 && V == 4)
            e = launch_maybe_dependent(true, batch_step_kernel_p_occ<S, V>, grid, block, 0, b->stream, b->params, step,
                                       reverse);
        else if constexpr (sizeof(S) <= 4)
            e = launch_maybe_dependent(true, batch_step_kernel_p<S, V>, grid, block, 0, b->stream, b->params, step,
                                       reverse);
        return e != cudaSuccess ? e : cudaGetLastError();
    }
    const SlotDesc *descs = b->desc_d;
    const Tile *tiles = b->tiles_d;
    if constexpr (sizeof(S) == 2 && V == 4)
        e = launch_maybe_dependent(true, batch_step_kernel_occ<S, V>, grid, block, 0, b->stream, descs, tiles,
                                   b->ntiles, step, reverse);
    else
        e = launch_maybe_dependent(true, batch_step_kernel<S, V>, grid, block, 0, b->stream, descs, tiles, b->ntiles,
                                   step, reverse);
    return e != cudaSuccess ? e : cudaGetLastError();
}

// mode 1: batches of at most this many live cells run a step sequence as one persistent launch.
// Measured on FP16 batches of 64^2-256^2 domains, 200-step sequences, against one launch per step:
// 1.48x at 2e4-7e4 cells, 1.05x at 3.8e5, 0.91x at 1.6e6 when every launch waited for the one
// before to drain; 0.82-0.87x at every size once each step launch is the programmatic dependent
// of the one before, hence mode 0 by default.
constexpr int64_t PERSIST_CELLS = (int64_t)1 << 19;

bool persistent_ok(const lbm_batch *b, int nsteps) {
    if (!b->use_params || b->v != 4 || nsteps < 2 || b->persist == 0) return false;
    return b->persist == 2 || b->live_cells <= PERSIST_CELLS;
}

template <class S>
cudaError_t launch_persistent_t(lbm_batch *b, int nsteps) {
    if constexpr (sizeof(S) > 4) {
        return cudaErrorInvalidValue;
    } else {
        const dim3 block(b->tx, b->ty);
        int per_sm = 0, sms = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_persistent_kernel<S>,
                                                                      (int)(block.x * block.y), 0);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorInvalidConfiguration;
        const int grid = std::min(b->ntiles, per_sm * sms);  // every block resident at once
        // arrivals from zero; the status word keeps a failure until lbm_batch_synchronize reads it
        e = cudaMemsetAsync(&b->sync_d->arrived, 0, sizeof(unsigned int), b->stream);
        if (e != cudaSuccess) return e;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = block;
        cfg.stream = b->stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, batch_persistent_kernel<S>, b->params, nsteps, (int)(b->sweep & 1u), b->sync_d,
                               b->persist_wait_ns, b->persist_skip);
        if (e == cudaSuccess) ++b->persist_launches;
        return e;
    }
}

cudaError_t launch_persistent(lbm_batch *b, int nsteps) {
    switch (b->dtype) {
        case LBM_F32: return launch_persistent_t<float>(b, nsteps);
        case LBM_F16S: return launch_persistent_t<__half>(b, nsteps);
        case LBM_BF16S: return launch_persistent_t<__nv_bfloat16>(b, nsteps);
    }
    return cudaErrorInvalidValue;
}

template <class S>
cudaError_t launch(lbm_batch *b, int step, int reverse) {
    if constexpr (vec_ok<S>(2)) {
        if (b->v == 2) return launch_v<S, 2>(b, step, reverse);
    }
    if constexpr (vec_ok<S>(4)) {
        if (b->v == 4) return launch_v<S, 4>(b, step, reverse);
    }
    if constexpr (vec_ok<S>(8)) {
        if (b->v == 8) return launch_v<S, 8>(b, step, reverse);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_any(lbm_batch *b, int step, int reverse) {
    switch (b->dtype) {
        case LBM_F32: return launch<float>(b, step, reverse);
        case LBM_F16S: return launch<__half>(b, step, reverse);
        case LBM_BF16S: return launch<__nv_bfloat16>(b, step, reverse);
        case LBM_F64: return launch<double>(b, step, reverse);
    }
    return cudaErrorInvalidValue;
}

// Time every candidate tile shape on the live batch (launches with the step parity kept even, so
// src -> dst is recomputed without changing the state), then the three fastest again with three
// times the launches, in forward and reverse order, and keep the fastest of those.
lbm_status tune(lbm_batch *b) {
    struct Cand {
        int v, tx, ty;
    };
    std::vector<Cand> cands;
    for (int v : {2, 4, 8})
        for (int tx : {32, 64, 128})
            for (int ty : {1, 2, 4, 8})
                if (shape_ok(b->dtype, v, tx, ty)) cands.push_back({v, tx, ty});
    if (cands.empty()) return bfail(b, LBM_ERR_UNSUPPORTED, "batch: no tile shape for this dtype");
    cudaEvent_t e0, e1;
    BCUDA(b, cudaEventCreate(&e0), "batch tune: event");
    BCUDA(b, cudaEventCreate(&e1), "batch tune: event");
    bool empty = false;
    // ms of n launches with tile shape c (after one warm-up launch); -1 when the batch is empty
    auto time_cand = [&](const Cand &c, int n, float &ms) -> lbm_status {
        ms = -1.0f;
        b->v = c.v;
        b->tx = c.tx;
        b->ty = c.ty;
        b->dirty = true;
        b->tiles_dirty = true;
        lbm_status st = rebuild(b, 1);
        if (st != LBM_OK) return st;
        if (b->ntiles == 0) {
            empty = true;
            return LBM_OK;
        }
        cudaError_t e = launch_any(b, 0, 0);
        if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
        for (int r = 0; r < n && e == cudaSuccess; ++r) e = launch_any(b, 0, r & 1);
        if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        BCUDA(b, e, "batch tune: launch");
        cudaEventElapsedTime(&ms, e0, e1);
        return LBM_OK;
    };
    std::vector<std::pair<float, Cand>> timed;
    lbm_status st = LBM_OK;
    for (const Cand &c : cands) {
        float ms;
        if ((st = time_cand(c, 4, ms)) != LBM_OK || empty) break;
        timed.push_back({ms, c});
    }
    Cand pick = cands[0];
    if (st == LBM_OK && !empty && !timed.empty()) {
        std::stable_sort(timed.begin(), timed.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
        const size_t top = std::min<size_t>(3, timed.size());
        std::vector<float> total(top, 0.0f);
        for (int pass = 0; pass < 2 && st == LBM_OK; ++pass)
            for (size_t k = 0; k < top && st == LBM_OK; ++k) {
                const size_t c = pass ? top - 1 - k : k;
                float ms;
                st = time_cand(timed[c].second, 12, ms);
                total[c] += ms;
            }
        pick = timed[0].second;
        float best = 1e30f;
        for (size_t k = 0; k < top; ++k)
            if (total[k] < best) {
                best = total[k];
                pick = timed[k].second;
            }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != LBM_OK) return st;
    b->v = pick.v;
    b->tx = pick.tx;
    b->ty = pick.ty;
    b->dirty = true;
    b->tiles_dirty = true;
    b->tuned = true;
    return LBM_OK;
}

// device staging for slot I/O, grown stream-ordered (work queued before keeps the old buffer)
lbm_status ensure_staging(lbm_batch *b, size_t bytes) {
    if (!b->result_d) BCUDA(b, cudaMallocAsync((void **)&b->result_d, 16 * sizeof(double), b->stream), "batch: result buffer");
    if (b->staging_bytes >= bytes) return LBM_OK;
    if (b->staging) cudaFreeAsync(b->staging, b->stream);
    b->staging = nullptr;
    b->staging_bytes = 0;
    BCUDA(b, cudaMallocAsync(&b->staging, bytes, b->stream), "batch: staging");
    b->staging_bytes = bytes;
    return LBM_OK;
}

Slot *get_slot(lbm_batch *b, int32_t slot) {
    if (!b || slot < 0 || (size_t)slot >= b->slots.size() || !b->slots[slot].live) return nullptr;
    return &b->slots[slot];
}



}  // namespace

extern "C" {

LBM_API lbm_status lbm_batch_create(int32_t dtype, int32_t device, void *stream, lbm_batch **out) {
    if (!out) return lbm::set_thread_error(LBM_ERR_INVALID, "null output");
    *out = nullptr;
    if (dsize(dtype) == 0 || dtype < LBM_F32 || dtype > LBM_F64) return lbm::set_thread_error(LBM_ERR_INVALID, "bad dtype");
    lbm_batch *b = new lbm_batch();
    b->dtype = dtype;
    b->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) {
        if (stream) {
            b->stream = static_cast<cudaStream_t>(stream);
        } else {
            e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
            b->own_stream = e == cudaSuccess;
        }
    }
    if (e != cudaSuccess) {
        delete b;
        return lbm::set_thread_error(LBM_ERR_CUDA, std::string("lbm_batch_create: ") + cudaGetErrorString(e));
    }
    // keep freed slot memory in the device's pool between requests instead of returning it to the
    // driver at every synchronisation
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
    default_shape(dtype, b->v, b->tx, b->ty);
    *out = b;
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_destroy(lbm_batch *b) {
    if (!b) return LBM_OK;
    cudaSetDevice(b->device);
    for (Slot &s : b->slots)
        if (s.live) free_slot(b, s);
    if (b->stream) cudaStreamSynchronize(b->stream);
    cudaFree(b->desc_d);
    cudaFree(b->tiles_d);
    cudaFree(b->sync_d);
    cudaFree(b->staging);
    cudaFree(b->result_d);
    for (PinnedBlock &pb : b->pinned) {
        cudaFreeHost(pb.p);
        cudaEventDestroy(pb.done);
    }
    if (b->own_stream) cudaStreamDestroy(b->stream);
    delete b;
    return LBM_OK;
}

LBM_API const char *lbm_batch_last_error(const lbm_batch *b) { return b ? b->err.c_str() : ""; }

LBM_API int64_t lbm_batch_slot_bytes(int32_t dtype, int32_t nx, int32_t ny) {
    if (nx < 1 || ny < 1 || dsize(dtype) == 0) return -1;
    const int64_t pitch = ((int64_t)nx + 31) / 32 * 32;
    return 2 * 9 * pitch * ny * (int64_t)dsize(dtype) + pitch * ny * 2 + (int64_t)flags_bytes(nx, ny);
}

LBM_API lbm_status lbm_batch_add(lbm_batch *b, const lbm_desc *desc, const uint8_t *host_flags, int32_t *slot_out) {
    if (!b || !desc || !slot_out) return bfail(b, LBM_ERR_INVALID, "lbm_batch_add: null argument");
    if (desc->mode != LBM_D2Q9 || desc->nz != 1 || desc->nx < 1 || desc->ny < 1)
        return bfail(b, LBM_ERR_INVALID, "lbm_batch_add: batches hold D2Q9 domains (nz = 1)");
    if (!(desc->tau > 0.5f)) return bfail(b, LBM_ERR_INVALID, "lbm_batch_add: tau must be > 0.5");
    if (desc->periodic < 0 || desc->periodic > 3) return bfail(b, LBM_ERR_INVALID, "lbm_batch_add: periodic must be 0..3");
    const int64_t pitch = ((int64_t)desc->nx + 31) / 32 * 32;
    if (pitch * desc->ny * 9 >= (int64_t)INT32_MAX) return bfail(b, LBM_ERR_INVALID, "lbm_batch_add: domain too large for a batch");
    BCUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    Slot s;
    s.desc = *desc;
    s.desc.dtype = b->dtype;
    s.pitch = (int)pitch;
    s.plane = pitch * desc->ny;
    const size_t pop = (size_t)s.plane * 9 * dsize(b->dtype);
    s.bytes = (size_t)lbm_batch_slot_bytes(b->dtype, desc->nx, desc->ny);
    auto cleanup = [&]() {
        free_slot(b, s);
        cudaStreamSynchronize(b->stream);
    };
    const size_t ncell = (size_t)desc->nx * desc->ny;
    // one allocation per slot: population buffers A and B, link words, flags and the fluid count
    // (the parameter-block kernel derives every pointer from the first)
    cudaError_t e = cudaMallocAsync(&s.f[0], 2 * pop + (size_t)s.plane * sizeof(uint16_t) + flags_bytes(desc->nx, desc->ny),
                                    b->stream);
    if (e == cudaSuccess) {
        char *base = static_cast<char *>(s.f[0]);
        s.f[1] = base + pop;
        s.links = reinterpret_cast<uint16_t *>(base + 2 * pop);
        s.flags = reinterpret_cast<uint8_t *>(base + 2 * pop + (size_t)s.plane * sizeof(uint16_t));
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return bfail(b, e == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA,
                     std::string("lbm_batch_add: ") + cudaGetErrorString(e));
    }
    s.live = true;
    s.count_d = reinterpret_cast<unsigned long long *>(s.flags + flags_bytes(desc->nx, desc->ny) - 8);
    // flags, link words, fluid count, equilibrium at rho = 1, u = 0 through the single-domain
    // kernels, all queued without waiting
    if (host_flags) {
        for (size_t i = 0; i < ncell; ++i)
            if (host_flags[i] > LBM_MOVING_WALL) {
                cleanup();
                return bfail(b, LBM_ERR_INVALID, "lbm_batch_add: flag values must be 0, 1 or 2");
            }
        if (upload_async(b, s.flags, host_flags, ncell, "lbm_batch_add: upload flags") != LBM_OK) {
            const std::string m = b->err;
            cleanup();
            return bfail(b, LBM_ERR_CUDA, m);
        }
    } else {
        e = cudaMemsetAsync(s.flags, 0, ncell, b->stream);
    }
    // link words of the row padding stay 0 (the vectorised step reads them)
    if (e == cudaSuccess) e = cudaMemsetAsync(s.links, 0, (size_t)s.plane * sizeof(uint16_t), b->stream);
    if (e == cudaSuccess) {
        CtxView v(b, s);
        e = d2q9_build_links_async(&v.c, s.count_d);
        if (e == cudaSuccess) e = d2q9_init_equilibrium(&v.c, nullptr, nullptr, nullptr);
    }
    if (e != cudaSuccess) {
        cleanup();
        return bfail(b, LBM_ERR_CUDA, std::string("lbm_batch_add: initialisation: ") + cudaGetErrorString(e));
    }
    int32_t id = -1;
    for (size_t i = 0; i < b->slots.size(); ++i)
        if (!b->slots[i].live) {
            id = (int32_t)i;
            break;
        }
    if (id < 0) {
        id = (int32_t)b->slots.size();
        b->slots.push_back(Slot());
    }
    b->slots[id] = s;
    b->device_bytes += (int64_t)s.bytes;
    b->live_cells += (int64_t)desc->nx * desc->ny;
    b->dirty = true;
    b->tiles_dirty = true;
    *slot_out = id;
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_remove(lbm_batch *b, int32_t slot) {
    Slot *s = get_slot(b, slot);
    if (!s) return bfail(b, LBM_ERR_INVALID, "lbm_batch_remove: no such slot");
    free_slot(b, *s);  // ordered after the queued steps that may still read the slot
    b->device_bytes -= (int64_t)s->bytes;
    b->live_cells -= (int64_t)s->desc.nx * s->desc.ny;
    *s = Slot();
    b->dirty = true;
    b->tiles_dirty = true;
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_set_launch(lbm_batch *b, int32_t cells_per_thread, int32_t block_threads,
                                        int32_t rows_per_block) {
    if (!b) return lbm::set_thread_error(LBM_ERR_INVALID, "null batch");
    if (!shape_ok(b->dtype, cells_per_thread, block_threads, rows_per_block))
        return bfail(b, LBM_ERR_INVALID, "lbm_batch_set_launch: shape not valid for this dtype");
    b->v = cells_per_thread;
    b->tx = block_threads;
    b->ty = rows_per_block;
    b->tuned = true;
    b->fixed = true;
    b->dirty = true;
    b->tiles_dirty = true;
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_autotune(lbm_batch *b) {
    if (!b) return lbm::set_thread_error(LBM_ERR_INVALID, "null batch");
    BCUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    b->fixed = false;
    lbm_status st = tune(b);
    if (st == LBM_OK) {
        b->tuned_cells = b->live_cells;
        ++b->tunings;
    }
    return st;
}

LBM_API lbm_status lbm_batch_tunings(lbm_batch *b, int32_t *count) {
    if (!b || !count) return lbm::set_thread_error(LBM_ERR_INVALID, "null argument");
    *count = b->tunings;
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_step(lbm_batch *b, int32_t nsteps) {
    if (!b) return lbm::set_thread_error(LBM_ERR_INVALID, "null batch");
    if (nsteps < 0) return bfail(b, LBM_ERR_INVALID, "nsteps must be >= 0");
    if (nsteps == 0) return LBM_OK;
    NvtxRange range("lbm_batch_step");
    BCUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    // Tuning on a handful of small slots would fix the shape for the mix that follows: the batch
    // keeps the default shape until it holds TUNE_CELLS cells, tunes then, and once more if it
    // grows to four times the cells it was tuned on.
    if (!b->fixed && b->live_cells >= TUNE_CELLS &&
        (!b->tuned || (b->tunings < 2 && b->live_cells >= 4 * b->tuned_cells))) {
        lbm_status st = tune(b);
        if (st != LBM_OK) return st;
        b->tuned_cells = b->live_cells;
        ++b->tunings;
    }
    lbm_status st = rebuild(b, nsteps);
    if (st != LBM_OK) return st;
    if (b->ntiles > 0) {
        bool done = false;
        if (persistent_ok(b, nsteps)) {
            if (!b->sync_d) BCUDA(b, cudaMalloc(&b->sync_d, sizeof(GridSync)), "batch: grid sync word");
            if (!b->sync_d_init) {
                BCUDA(b, cudaMemsetAsync(b->sync_d, 0, sizeof(GridSync), b->stream), "batch: grid sync word");
                b->sync_d_init = true;
            }
            BCUDA(b, launch_persistent(b, nsteps), "batch persistent launch");
            done = true;
        }
        for (int s = 0; !done && s < nsteps; ++s) {
            BCUDA(b, launch_any(b, s, (int)((b->sweep + s) & 1)), "batch step");
        }
    }
    b->sweep += (unsigned)nsteps;
    // each live slot advanced by its own count: its current buffer moves on by that parity
    for (Slot &s : b->slots)
        if (s.live) {
            const int64_t adv = advance_of(s, nsteps);
            s.cur = (int)((s.cur + adv) & 1);
            s.steps_done += adv;
            if (s.limit >= 0) s.limit -= adv;
            if (adv & 1) b->dirty = true;  // descriptors carry the parity
        }
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_set_slot_steps(lbm_batch *b, int32_t slot, int64_t steps) {
    Slot *s = get_slot(b, slot);
    if (!s) return bfail(b, LBM_ERR_INVALID, "lbm_batch_set_slot_steps: no such slot");
    s->limit = steps < 0 ? -1 : steps;
    b->dirty = true;
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_synchronize(lbm_batch *b) {
    if (!b) return lbm::set_thread_error(LBM_ERR_INVALID, "null batch");
    BCUDA(b, cudaStreamSynchronize(b->stream), "batch synchronize");
    if (b->sync_d) {
        unsigned int status = 0;
        BCUDA(b, cudaMemcpy(&status, &b->sync_d->status, sizeof(status), cudaMemcpyDeviceToHost), "batch synchronize");
        if (status) {
            BCUDA(b, cudaMemset(&b->sync_d->status, 0, sizeof(status)), "batch synchronize");
            return bfail(b, LBM_ERR_TIMEOUT,
                         "batch: a persistent launch gave up waiting for its blocks; the slots' populations are "
                         "not valid");
        }
    }
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_set_persistent(lbm_batch *b, int32_t mode, int64_t wait_ns, int32_t skip_block) {
    if (!b) return lbm::set_thread_error(LBM_ERR_INVALID, "null batch");
    if (mode < 0 || mode > 2) return bfail(b, LBM_ERR_INVALID, "lbm_batch_set_persistent: mode must be 0, 1 or 2");
    if (wait_ns <= 0) return bfail(b, LBM_ERR_INVALID, "lbm_batch_set_persistent: wait_ns must be > 0");
    b->persist = mode;
    b->persist_wait_ns = wait_ns;
    b->persist_skip = skip_block;
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_get_stream(lbm_batch *b, void **stream) {
    if (!b || !stream) return lbm::set_thread_error(LBM_ERR_INVALID, "null argument");
    *stream = b->stream;
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_info(lbm_batch *b, int64_t out[8]) {
    if (!b || !out) return lbm::set_thread_error(LBM_ERR_INVALID, "null argument");
    int64_t live = 0, cells = 0, fluid = 0;
    for (Slot &s : b->slots)
        if (s.live && s.fluid < 0) {  // read the counts queued by lbm_batch_add
            unsigned long long h = 0;
            BCUDA(b, cudaMemcpyAsync(&h, s.count_d, sizeof(h), cudaMemcpyDeviceToHost, b->stream), "batch info");
            BCUDA(b, cudaStreamSynchronize(b->stream), "batch info");
            s.fluid = (int64_t)h;
        }
    for (const Slot &s : b->slots)
        if (s.live) {
            ++live;
            cells += (int64_t)s.desc.nx * s.desc.ny;
            fluid += s.fluid;
        }
    out[0] = live;
    out[1] = cells;
    out[2] = fluid;
    out[3] = b->device_bytes;
    out[4] = b->v;
    out[5] = b->tx;
    out[6] = b->ty;
    out[7] = b->ntiles;
    return LBM_OK;
}

// Per-slot host I/O through the single-domain conversion kernels on a view of the slot.
// Moments: density and velocity into device staging, then into a pinned block, queued; the ticket
// is collected (copied into the caller's arrays) once the copy has completed.
LBM_API lbm_status lbm_batch_moments_async(lbm_batch *b, int32_t slot, int64_t *ticket) {
    Slot *s = get_slot(b, slot);
    if (!s || !ticket) return bfail(b, LBM_ERR_INVALID, "lbm_batch_moments_async: no such slot or null ticket");
    BCUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    const size_t n = (size_t)s->desc.nx * s->desc.ny;
    lbm_status st = ensure_staging(b, 3 * n * sizeof(float));
    if (st != LBM_OK) return st;
    float *buf = static_cast<float *>(b->staging);
    size_t k;
    if ((st = pinned_get(b, 3 * n * sizeof(float), &k)) != LBM_OK) return st;
    CtxView v(b, *s);
    cudaError_t e = d2q9_moments(&v.c, buf, buf + n, buf + 2 * n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->pinned[k].p, buf, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->pinned[k].done, b->stream);
    BCUDA(b, e, "lbm_batch_moments_async");
    const int64_t id = b->next_ticket++;
    b->pending[id] = Pending{k, n, b->pinned[k].done};
    *ticket = id;
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_collect(lbm_batch *b, int64_t ticket, int32_t wait, float *rho, float *ux, float *uy,
                                     int32_t *ready) {
    if (!b || !ready) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_batch_collect: null argument");
    auto it = b->pending.find(ticket);
    if (it == b->pending.end()) return bfail(b, LBM_ERR_INVALID, "lbm_batch_collect: no such ticket");
    *ready = 0;
    const Pending pd = it->second;
    if (wait) {
        BCUDA(b, cudaEventSynchronize(pd.done), "lbm_batch_collect");
    } else {
        const cudaError_t q = cudaEventQuery(pd.done);
        if (q == cudaErrorNotReady) {
            cudaGetLastError();
            return LBM_OK;
        }
        BCUDA(b, q, "lbm_batch_collect");
    }
    const float *src = static_cast<const float *>(b->pinned[pd.block].p);
    float *host[3] = {rho, ux, uy};
    for (int c = 0; c < 3; ++c)
        if (host[c]) std::memcpy(host[c], src + c * pd.n, pd.n * sizeof(float));
    b->pending.erase(it);
    *ready = 1;
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_moments(lbm_batch *b, int32_t slot, float *rho, float *ux, float *uy) {
    int64_t ticket = 0;
    lbm_status st = lbm_batch_moments_async(b, slot, &ticket);
    if (st != LBM_OK) return st;
    int32_t ready = 0;
    return lbm_batch_collect(b, ticket, 1, rho, ux, uy, &ready);
}

LBM_API lbm_status lbm_batch_retrieve_populations(lbm_batch *b, int32_t slot, void *host, int32_t host_dtype) {
    Slot *s = get_slot(b, slot);
    if (!s || !host || (host_dtype != LBM_F32 && host_dtype != LBM_F64))
        return bfail(b, LBM_ERR_INVALID, "lbm_batch_retrieve_populations: bad arguments");
    BCUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    const size_t bytes = (size_t)s->desc.nx * s->desc.ny * 9 * (host_dtype == LBM_F64 ? 8 : 4);
    lbm_status st = ensure_staging(b, bytes);
    if (st != LBM_OK) return st;
    void *buf = b->staging;
    CtxView v(b, *s);
    cudaError_t e = d2q9_store(&v.c, buf, host_dtype, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, buf, bytes, cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    BCUDA(b, e, "lbm_batch_retrieve_populations");
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_load_populations(lbm_batch *b, int32_t slot, const void *host, int32_t host_dtype) {
    Slot *s = get_slot(b, slot);
    if (!s || !host || (host_dtype != LBM_F32 && host_dtype != LBM_F64))
        return bfail(b, LBM_ERR_INVALID, "lbm_batch_load_populations: bad arguments");
    BCUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    const size_t bytes = (size_t)s->desc.nx * s->desc.ny * 9 * (host_dtype == LBM_F64 ? 8 : 4);
    lbm_status st = ensure_staging(b, bytes);
    if (st != LBM_OK) return st;
    void *buf = b->staging;
    CtxView v(b, *s);
    cudaError_t e = cudaMemcpyAsync(buf, host, bytes, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = d2q9_load(&v.c, buf, host_dtype, 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    BCUDA(b, e, "lbm_batch_load_populations");
    return LBM_OK;
}

LBM_API lbm_status lbm_batch_slot_steps(lbm_batch *b, int32_t slot, int64_t *steps_done) {
    Slot *s = get_slot(b, slot);
    if (!s || !steps_done) return bfail(b, LBM_ERR_INVALID, "lbm_batch_slot_steps: bad arguments");
    *steps_done = s->steps_done;
    return LBM_OK;
}

}  // extern "C"
