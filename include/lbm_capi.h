/*
 * lbm_capi.h -- C ABI of the GB300 lattice Boltzmann library (liblbm_gb300.so).
 *
 * This is the drop-in boundary for the reference's collide-stream path.  The reference exposes
 * that path as the C++ class Lattice (simulation/include/Lattice.h:40-106) on top of the launch
 * wrappers RunCudaFunctions::run_* (simulation/include/SimCalcFuncs.cuh:13-25); a C++
 * compatibility layer with those names is built on this ABI (latticeboltzmanncuda_gb300/compat:
 * liblbm_compat.so and the reference's command line), and other languages bind these functions
 * directly (ctypes, cgo, JNI).
 *
 * Conventions
 *   - Every function returns an lbm_status; lbm_last_error() gives the message of the last
 *     failure on a context (or, for a NULL context, of the calling thread).
 *   - Plain pointers and sizes only.  Pointers named host_* are host memory owned by the caller;
 *     the context owns all device memory it allocates and frees it in lbm_destroy().
 *   - One context per host thread at a time.  Each context works on its own CUDA stream (the one
 *     given in lbm_desc.stream, or a non-blocking stream it creates).  Functions that read results
 *     back to the host synchronise that stream; lbm_step() only enqueues work.
 *   - Two lattice modes share the API:
 *       LBM_D2Q9      standard D2Q9 BGK: pull streaming, half-way bounce-back, moving walls,
 *                     periodic edges, Guo body force; populations stored shifted (f_i - w_i) in
 *                     FP32, FP16, BF16 or FP64.
 *       LBM_D3Q27_REF the reference's own D3Q27 step (SimCalcFuncs.cu:79-215): zero-fill pull
 *                     streaming, mesh "reflections", SPLIT-weighted velocity, FP64-evaluated
 *                     equilibrium, mass-source flow; FP32 populations.
 */
#ifndef LBM_CAPI_H
#define LBM_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define LBM_API __attribute__((visibility("default")))
#else
#define LBM_API
#endif

typedef enum lbm_status {
    LBM_OK = 0,
    LBM_ERR_INVALID = 1,     /* bad argument or size */
    LBM_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    LBM_ERR_OOM = 3,         /* device allocation failed */
    LBM_ERR_UNSUPPORTED = 4, /* call not available in this mode / dtype */
    LBM_ERR_STATE = 5,       /* call out of order (e.g. step before flags) */
    LBM_ERR_BUDGET = 6,      /* request does not fit the server's memory budget */
    LBM_ERR_TIMEOUT = 7      /* a bounded wait gave up */
} lbm_status;

typedef enum lbm_mode { LBM_D2Q9 = 0, LBM_D3Q27_REF = 1 } lbm_mode;

typedef enum lbm_dtype {
    LBM_F32 = 0,   /* FP32 storage (D2Q9: shifted f_i - w_i) */
    LBM_F16S = 1,  /* FP16 storage of f_i - w_i, FP32 arithmetic (D2Q9 only) */
    LBM_BF16S = 2, /* BF16 storage of f_i - w_i, FP32 arithmetic (D2Q9 only) */
    LBM_F64 = 3    /* FP64 storage and arithmetic: the GPU oracle run (D2Q9 only) */
} lbm_dtype;

/* D2Q9 cell flags (one byte per cell, row-major [ny][nx]) */
enum { LBM_FLUID = 0, LBM_WALL = 1, LBM_MOVING_WALL = 2 };

/* D3Q27_REF cell flag bits (one byte per cell, reference index z + Z*(y + Y*x)):
 * LatticePoint::isInternal, LatticePoint::isReflected (LatticePoint.h:13-14) and the flow
 * criterion of FlowData (FlowSurface.h:9-46) evaluated once per cell. */
enum { LBM_INTERNAL = 1, LBM_REFLECTED = 2, LBM_SOURCE = 4 };

/* D3Q27_REF step orders for lbm_step():
 *   LBM_ORDER_STREAM_COLLIDE  Lattice::simulateLattice (Lattice.cpp:222-226)
 *   LBM_ORDER_CLI             stream, reflect, collide, flow (LatticeBoltzmannCuda.cpp:85-93) */
enum { LBM_ORDER_STREAM_COLLIDE = 0, LBM_ORDER_CLI = 1 };

/* D3Q27_REF single passes for lbm_apply(), one flag per call (Lattice::simulateStreaming,
 * simulateReflections, simulateCollision, simulateFlow; Lattice.cpp:115-220) */
enum { LBM_OP_STREAM = 1, LBM_OP_REFLECT = 2, LBM_OP_COLLIDE = 4, LBM_OP_FLOW = 8 };

/* D3Q27_REF momentum-exchange force convention (SimCalcFuncs.cu:179-184):
 *   LBM_FORCE_REFERENCE          the reference's slot-indexed term c_s*SPLIT[s] (slots >= 27,
 *                                undefined in the reference, contribute no incoming term)
 *   LBM_FORCE_MOMENTUM_EXCHANGE  the arriving population's term c_{s/3}*SPLIT[s/3] */
enum { LBM_FORCE_REFERENCE = 0, LBM_FORCE_MOMENTUM_EXCHANGE = 1 };

typedef struct lbm_desc {
    int32_t mode;             /* lbm_mode */
    int32_t dtype;            /* lbm_dtype */
    int32_t nx, ny, nz;       /* D2Q9: nx x ny (nz = 1); D3Q27_REF: X, Y, Z of Lattice(x, y, z, ...) */
    int32_t periodic;         /* D2Q9: bit0 periodic in x, bit1 periodic in y; other edges are walls */
    float tau;                /* relaxation time (FluidData::m_characteristicTimescale) */
    float body_force[3];      /* D2Q9: Guo body force per cell (x, y) */
    float wall_velocity[3];   /* D2Q9: velocity of LBM_MOVING_WALL cells (x, y) */
    int32_t order;            /* D3Q27_REF: LBM_ORDER_* used by lbm_step() */
    int32_t force_mode;       /* D3Q27_REF: LBM_FORCE_* */
    int32_t device;           /* CUDA device ordinal */
    void *stream;             /* cudaStream_t to work on, or NULL for a private stream */
} lbm_desc;

typedef struct lbm_ctx lbm_ctx;

typedef struct lbm_info {
    int64_t cells;            /* nx*ny*nz */
    int64_t fluid_cells;      /* D2Q9: cells with LBM_FLUID after lbm_set_flags() */
    int64_t row_pitch;        /* D2Q9: elements per stored row (nx rounded up) */
    int64_t state_bytes;      /* device bytes of both population buffers */
    int64_t device_bytes;     /* all device bytes owned by the context */
    int64_t bytes_per_update; /* algorithmic bytes per cell update: 2 * Q * sizeof(storage) */
    int64_t steps_done;
    int32_t block_threads;    /* D2Q9 step kernel launch shape: threads along x per block, */
    int32_t cells_per_thread; /* consecutive cells per thread (0: bulk-copy pipeline; -2, -3: two */
    int32_t rows_per_block;   /* steps per launch on tiles of block_threads x rows_per_block cells), */
                              /* rows per block */
    int32_t tuned;            /* 1 once the shape has been chosen */
    int32_t l2_policy;        /* L2 eviction hints of the vectorised path (see lbm_set_launch) */
} lbm_info;

/* ---------------------------------------------------------------- context life cycle */
LBM_API void lbm_desc_init(lbm_desc *desc);
LBM_API lbm_status lbm_create(const lbm_desc *desc, lbm_ctx **out);
LBM_API lbm_status lbm_destroy(lbm_ctx *ctx);
LBM_API const char *lbm_last_error(const lbm_ctx *ctx);
LBM_API const char *lbm_status_string(lbm_status s);
LBM_API lbm_status lbm_get_info(lbm_ctx *ctx, lbm_info *out);
LBM_API lbm_status lbm_get_stream(lbm_ctx *ctx, void **stream);
LBM_API lbm_status lbm_synchronize(lbm_ctx *ctx);
/* change tau / body force / wall velocity between steps */
LBM_API lbm_status lbm_set_params(lbm_ctx *ctx, float tau, const float body_force[3],
                                  const float wall_velocity[3]);

/* ---------------------------------------------------------------- geometry and state */
/* Cell flags, host_flags[cells] (layout per mode, see enums above).  Replaces
 * Lattice::insertModel's isInternal output (Lattice.cpp:228-260) for D3Q27_REF. */
LBM_API lbm_status lbm_set_flags(lbm_ctx *ctx, const uint8_t *host_flags);
LBM_API lbm_status lbm_get_flags(lbm_ctx *ctx, uint8_t *host_flags);

/* D2Q9: populations = equilibrium of (rho, ux, uy) per cell; NULL arrays mean rho = 1, u = 0. */
LBM_API lbm_status lbm_init_equilibrium(lbm_ctx *ctx, const float *host_rho, const float *host_ux,
                                        const float *host_uy);

/* Raw populations, unshifted, as float (host_dtype LBM_F32) or double (LBM_F64).
 *   D2Q9:      host[q][ny][nx], q in the order (0,0),(1,0),(0,1),(-1,0),(0,-1),(1,1),(-1,1),
 *              (-1,-1),(1,-1)
 *   D3Q27_REF: host[cell][27] in the reference's particle_distribution order (SimCalcFuncs.cu:12) */
LBM_API lbm_status lbm_load_populations(lbm_ctx *ctx, const void *host, int32_t host_dtype);
LBM_API lbm_status lbm_retrieve_populations(lbm_ctx *ctx, void *host, int32_t host_dtype);

/* Reference AoS records (struct LatticePoint, LatticePoint.h:9-17, 144 bytes each), count =
 * cells, record index z + Z*(y + Y*x); 2-D lattices use X = nx, Y = ny, Z = 1 and the in-plane
 * slots {0,6,5,1,2,18,10,7,15} for the D2Q9 populations.  Replaces Lattice::load_data /
 * retrieve_data (Lattice.cpp:73-113).  Loading takes particle_distribution and, in D3Q27_REF,
 * isInternal / isReflected; retrieving writes x, y, z, particle_distribution and the flags and
 * sets both reflection pointers to NULL. */
LBM_API lbm_status lbm_load_aos(lbm_ctx *ctx, const void *host_points, int64_t count);
LBM_API lbm_status lbm_retrieve_aos(lbm_ctx *ctx, void *host_points, int64_t count);

/* D3Q27_REF reflection tables: records[i] (struct ReflectionValues, LatticePoint.h:3-7,
 * 380 bytes) belongs to cell cells[i] (reference index).  Replaces the device upload of
 * Lattice::preProcessModel (Lattice.cpp:417-423).  count = 0 clears the tables. */
LBM_API lbm_status lbm_set_reflection_tables(lbm_ctx *ctx, int64_t count, const int32_t *host_cells,
                                             const void *host_records);

/* D3Q27_REF flow source (FlowData, FlowSurface.h:9-46; Lattice::setFlowData, Lattice.cpp:428-436):
 * host_mask[cells] != 0 marks cells where the criterion holds (NULL keeps the current mask),
 * host_induced[27] the populations added there each step (NULL disables flow). */
LBM_API lbm_status lbm_set_flow(lbm_ctx *ctx, const uint8_t *host_mask, const float *host_induced);

/* D3Q27_REF accumulated momentum-exchange force (ReflectionData, Lattice.h:33-38).
 * lbm_set_force starts accumulation from host_in (Lattice::setReflectionData, Lattice.cpp:61-71);
 * enabled = 0 stops accumulating.  lbm_get_force reads the running sum
 * (Lattice::retrieve_reflection_data, Lattice.cpp:438-443). */
LBM_API lbm_status lbm_set_force(lbm_ctx *ctx, const float host_in[3], int32_t enabled);
LBM_API lbm_status lbm_get_force(lbm_ctx *ctx, float host_out[3]);
/* Turn accumulation on or off keeping the running sum (the reference's plain reflection pass,
 * run_calculate_reflections, adds no force); lbm_force_accumulation reports the current state. */
LBM_API lbm_status lbm_set_force_accumulation(lbm_ctx *ctx, int32_t enabled);
LBM_API int32_t lbm_force_accumulation(const lbm_ctx *ctx);

/* ---------------------------------------------------------------- stepping */
/* Advance nsteps fused time steps (one read and one write of the populations per step). */
LBM_API lbm_status lbm_step(lbm_ctx *ctx, int32_t nsteps);
/* D3Q27_REF: one separate pass (LBM_OP_*), as the reference's Lattice::simulate* methods. */
LBM_API lbm_status lbm_apply(lbm_ctx *ctx, int32_t op);
/* D3Q27_REF equilibrium evaluation.  The reference evaluates eq_i in FP64 and rounds it to FP32
 * (SimCalcFuncs.cu:122-155).  The first two modes give that value bit for bit:
 *   LBM_EQ_FLOAT_FLOAT (default)  float-float arithmetic with a proven error bound, falling back to
 *                                 the FP64 expression when the bound cannot decide the FP32 rounding
 *   LBM_EQ_FP64                   the FP64 expression for every direction (GB300's FP64 rate bounds
 *                                 the step)
 *   LBM_EQ_FP32                   the same expression in FP32 (a few ulps from the FP64 value; the
 *                                 populations stay within 1e-5 relative of the reference's), for
 *                                 speed. */
enum { LBM_EQ_FLOAT_FLOAT = 0, LBM_EQ_FP64 = 1, LBM_EQ_FP32 = 2 };
LBM_API lbm_status lbm_set_equilibrium_evaluation(lbm_ctx *ctx, int32_t mode);
/* Diagnostic: both evaluations on `samples` pseudo-random (rho, u) draws (|u| up to 2) x the 27
 * directions on `device`; out[0] = float-float results accepted by their bound that differ from
 * FP64 (must be 0), out[1] = direction pairs left to the FP64 fallback among the draws with
 * |u| <= 0.05. */
LBM_API lbm_status lbm_d3q27_equilibrium_selftest(int64_t samples, uint64_t seed, int32_t device, int64_t out[2]);
/* Diagnostic: the D3Q27_REF step divides by tau with one correction of RN(x * RN(1/tau))
 * (Markstein 1990) where that equals the IEEE division; this counts, over all 2^32 float inputs x,
 * the quotients that would differ for this tau (the library checks each tau it uses the same way
 * and keeps the IEEE division for a tau with any difference). */
LBM_API lbm_status lbm_d3q27_division_check(float tau, int32_t device, int64_t *mismatches);
/* D3Q27_REF: the step order of later lbm_step() calls (LBM_ORDER_*), e.g. the stream-collide of
 * Lattice::simulateLattice and the CLI loop on one lattice. */
LBM_API lbm_status lbm_set_order(lbm_ctx *ctx, int32_t order);
/* D3Q27_REF: lbm_step(nsteps) that also records the accumulated force after every step,
 * host_series[3*s + k] = component k after step s + 1, with one device-to-host copy at the end.
 * Replaces the force print of the reference CLI loop (LatticeBoltzmannCuda.cpp:78-93), which
 * copies ReflectionData back and synchronises once per step. */
LBM_API lbm_status lbm_step_force_series(lbm_ctx *ctx, int32_t nsteps, float *host_series);

/* D2Q9 launch shape.  The first lbm_step() picks it with a built-in autotuner: every candidate
 * (cells per thread 1/2/4/8 as the storage type allows, block widths 32..256, 1..4 rows per block)
 * is timed on the context's own domain, leaving the state unchanged, and the fastest is kept,
 * cached per (dtype, size, periodicity, force) in the process and in the JSON file named by
 * $LBM_TUNE_CACHE (default ~/.cache/lbm_gb300_tune.json; empty: no file).  LBM_AUTOTUNE=0 skips the
 * timing and uses a fixed default shape.  lbm_autotune() runs the tuner now (retune != 0 ignores the
 * caches); lbm_set_launch() fixes a shape (cells_per_thread in 1,2,4,8; block_threads a multiple of
 * 32; block_threads * rows_per_block <= 256) and the L2 eviction hints of the vectorised path
 * (l2_policy 0: none; 1: loads evict-first, stores evict-last; 2: loads evict-first; the scalar
 * path, cells_per_thread 1, takes 0 only).  cells_per_thread 0 selects the bulk-copy pipeline of
 * FP16/BF16 storage: persistent blocks of block_threads = 160 threads (rows_per_block = 1), one
 * warp staging the populations each row of a 512-cell strip pulls into a ring of shared-memory
 * slots with cp.async.bulk, four warps updating the rows; for it l2_policy selects the ring (0: 4
 * slots and 5 blocks per SM, 1: 4 slots and 4 blocks, 2: 6 slots and 3 blocks).  Its waits are
 * bounded: if one gives up, the next call that synchronises the context returns LBM_ERR_TIMEOUT.
 * cells_per_thread -2 selects two time steps per launch on shared-memory tiles of block_threads x
 * rows_per_block cells (64 x 8, 64 x 16 or 128 x 8; l2_policy 0; FP32 and 16-bit storage): each
 * block loads its tile with a two-cell halo, computes the first step on the tile grown by one cell
 * and the second into the destination, so the populations cross HBM once per two updates (an odd
 * last step of a call runs the one-step kernel).  cells_per_thread -3 is the same with persistent
 * blocks (64 x 4 or 64 x 8 tiles) that copy the next tile into a second buffer by cp.async while
 * they compute the current one.  Every shape gives bit-identical populations. */
LBM_API lbm_status lbm_autotune(lbm_ctx *ctx, int32_t retune);
LBM_API lbm_status lbm_set_launch(lbm_ctx *ctx, int32_t cells_per_thread, int32_t block_threads,
                                  int32_t rows_per_block, int32_t l2_policy);
/* D2Q9: visit rows in alternating order on successive steps (default 1), so each step starts on
 * the rows that the previous step wrote last and that are still in L2. */
LBM_API lbm_status lbm_set_sweep_alternation(lbm_ctx *ctx, int32_t enabled);
/* D2Q9 bulk-copy pipeline (cells_per_thread 0): every wait of its blocks gives up after wait_ns
 * nanoseconds (default 1e9; 1e3..1e10).  Diagnostic: skip_task >= 0 makes the copying warp leave
 * out the copies of that (strip, row) task in every launch, so the wait for them gives up: the next
 * call that synchronises the context returns LBM_ERR_TIMEOUT and the populations of the steps since
 * the previous synchronisation are not valid (reload them).  skip_task = -1 (the default) copies
 * every task.  No counterpart in the reference, whose kernels have no waits. */
LBM_API lbm_status lbm_set_pipeline_wait(lbm_ctx *ctx, int64_t wait_ns, int32_t skip_task);

/* ---------------------------------------------------------------- results */
/* Density and velocity per cell (host arrays of cells floats, any may be NULL).
 * D2Q9: moments of the streamed populations with the half-force shift (solid cells: rho = 1,
 * u = 0).  D3Q27_REF: density and the reference's SPLIT-weighted velocity of the stored
 * populations (SimCalcFuncs.cu:107-120). */
LBM_API lbm_status lbm_moments(lbm_ctx *ctx, float *host_rho, float *host_ux, float *host_uy,
                               float *host_uz);
/* FP64 sums over non-solid cells of the stored populations: mass, momentum x, y, z. */
LBM_API lbm_status lbm_conservation(lbm_ctx *ctx, double host_out[4]);

/* ---------------------------------------------------------------- checkpoint and resume */
/* No counterpart in the reference, whose only host snapshot is Lattice::retrieve_data / load_data
 * (Lattice.cpp:73-113, the populations alone).  lbm_save writes the context's state to a file: the
 * descriptor (size, storage type, tau, force, wall velocity, periodicity, step order, force mode),
 * the step count, the cell flags, the current populations in their storage type and device layout
 * (so a resumed run continues bit for bit), and for D3Q27_REF the reflection tables, the flow
 * source, the accumulated force and the equilibrium evaluation.  lbm_load restores it into a
 * context of the same mode, storage type and size (the other descriptor fields are taken from the
 * file); lbm_checkpoint_desc reads a file's descriptor, to create such a context.  The file is
 * written to path + ".tmp" and renamed; a checksum guards the payload.  Host byte order. */
LBM_API lbm_status lbm_save(lbm_ctx *ctx, const char *path);
LBM_API lbm_status lbm_load(lbm_ctx *ctx, const char *path);
LBM_API lbm_status lbm_checkpoint_desc(const char *path, lbm_desc *out);

/* ---------------------------------------------------------------- batched domains */
/* Many independent D2Q9 domains ("slots": own size, tau, force, wall velocity, periodicity and
 * flags) advanced together, one kernel launch per time step for all live slots (small batches: one
 * persistent launch per step sequence, see lbm_batch_set_persistent).  No counterpart
 * in the reference, which runs one lattice per process; each slot computes exactly what a
 * single-domain context with the same descriptor computes (bit-identical populations).  Slots
 * are added (allocated, flags set, equilibrium rho = 1, u = 0) and removed between steps;
 * lbm_batch_step advances every live slot.  The tile shape (cells per thread, block width, rows
 * per block) is tuned on the batch itself by the first lbm_batch_step that finds 2^24 or more live
 * cells (until then a default shape runs), and once more when the live cells have grown to four
 * times those it was tuned on; lbm_batch_autotune tunes now, lbm_batch_set_launch fixes a shape.
 * Adding, removing and stepping only queue work on the batch stream (host data is staged through
 * pinned memory), so a request loop can prepare its next round while the device runs the current
 * one; device errors of queued work surface at the next call that waits (lbm_batch_synchronize,
 * lbm_batch_collect with wait, lbm_batch_moments, lbm_batch_info). */
typedef struct lbm_batch lbm_batch;
LBM_API lbm_status lbm_batch_create(int32_t dtype, int32_t device, void *stream, lbm_batch **out);
LBM_API lbm_status lbm_batch_destroy(lbm_batch *b);
LBM_API const char *lbm_batch_last_error(const lbm_batch *b);
/* device bytes a slot of this size takes (two population buffers, link words, flags and the
 * fluid-cell count) */
LBM_API int64_t lbm_batch_slot_bytes(int32_t dtype, int32_t nx, int32_t ny);
/* desc: mode LBM_D2Q9, nx, ny, tau, periodic, body_force, wall_velocity (dtype, device and stream
 * come from the batch); host_flags[ny][nx] may be NULL (all fluid) */
LBM_API lbm_status lbm_batch_add(lbm_batch *b, const lbm_desc *desc, const uint8_t *host_flags,
                                 int32_t *slot_out);
LBM_API lbm_status lbm_batch_remove(lbm_batch *b, int32_t slot);
LBM_API lbm_status lbm_batch_step(lbm_batch *b, int32_t nsteps);
LBM_API lbm_status lbm_batch_autotune(lbm_batch *b);
/* how many times the batch has tuned its tile shape */
LBM_API lbm_status lbm_batch_tunings(lbm_batch *b, int32_t *count);
LBM_API lbm_status lbm_batch_set_launch(lbm_batch *b, int32_t cells_per_thread, int32_t block_threads,
                                        int32_t rows_per_block);
/* Waits for the batch stream; LBM_ERR_TIMEOUT when a persistent launch (below) gave up waiting for
 * its blocks since the last call (the slots' populations are then not valid). */
LBM_API lbm_status lbm_batch_synchronize(lbm_batch *b);
/* Persistent launches: a step sequence of lbm_batch_step (two steps or more) runs as one
 * cooperative launch whose blocks meet after each step, instead of one launch per step.  With
 * 4-wide tiles (the default shape of batches below the tuning threshold), for FP32 and 16-bit
 * storage.  mode 0 (default): never; 1: batches of at most 2^19 live cells; 2: whenever the shape
 * allows.  One launch per step, each launch allowed to start while the one before finishes, measured
 * faster than the persistent launch on batches of 2e4 to 1.6e6 cells.  Each meeting waits at most wait_ns
 * (default 1e9) for the other blocks, then the launch ends and lbm_batch_synchronize reports
 * LBM_ERR_TIMEOUT.  skip_block >= 0 is a diagnostic: that block does not arrive at the first
 * meeting, so the wait runs out (no counterpart in the reference). */
LBM_API lbm_status lbm_batch_set_persistent(lbm_batch *b, int32_t mode, int64_t wait_ns, int32_t skip_block);
LBM_API lbm_status lbm_batch_get_stream(lbm_batch *b, void **stream);
/* out: live slots, cells, fluid cells, device bytes of the slots, cells per thread, block width,
 * rows per block, tiles per step */
LBM_API lbm_status lbm_batch_info(lbm_batch *b, int64_t out[8]);
LBM_API lbm_status lbm_batch_slot_steps(lbm_batch *b, int32_t slot, int64_t *steps_done);
/* step budget of a slot: lbm_batch_step advances it by min(nsteps, budget) and lowers the budget;
 * a slot whose budget runs out mid-sequence stops there (-1: no budget, the default) */
LBM_API lbm_status lbm_batch_set_slot_steps(lbm_batch *b, int32_t slot, int64_t steps);
LBM_API lbm_status lbm_batch_moments(lbm_batch *b, int32_t slot, float *host_rho, float *host_ux,
                                     float *host_uy);
/* The same read-back queued without waiting: *ticket names it.  The slot may be removed right
 * after.  lbm_batch_collect copies a ticket's density and velocity into the host arrays (any may
 * be NULL) and releases it; with wait == 0 it returns at once with *ready = 0 while the copy is
 * still running. */
LBM_API lbm_status lbm_batch_moments_async(lbm_batch *b, int32_t slot, int64_t *ticket);
LBM_API lbm_status lbm_batch_collect(lbm_batch *b, int64_t ticket, int32_t wait, float *host_rho,
                                     float *host_ux, float *host_uy, int32_t *ready);
LBM_API lbm_status lbm_batch_load_populations(lbm_batch *b, int32_t slot, const void *host,
                                              int32_t host_dtype);
LBM_API lbm_status lbm_batch_retrieve_populations(lbm_batch *b, int32_t slot, void *host,
                                                  int32_t host_dtype);

/* ---------------------------------------------------------------- serving */
/* Continuous-batching solve server.  No counterpart in the reference.  lbm_server_run plays a
 * list of solve requests with arrival times in real time: requests wait in arrival order and are
 * admitted when their device bytes (lbm_batch_slot_bytes) fit into budget_bytes next to the live
 * solves and fewer than max_slots run (0: no slot limit); every round advances all live solves by
 * up to round_steps steps in one lbm_batch, so requests that arrive meanwhile join at the next
 * round and their work overlaps with the running ones.  A finished solve's density and velocity
 * go to the request's host buffers (if given) and its memory is released.  Per request: status
 * (LBM_OK; LBM_ERR_BUDGET if it alone exceeds the budget; LBM_ERR_INVALID; LBM_ERR_TIMEOUT if
 * time_limit seconds passed first), admission and completion times.  Each solve's result is
 * bit-identical to the same solve run alone. */
typedef struct lbm_server lbm_server;
typedef struct lbm_server_config {
    int32_t dtype;          /* storage type of every solve (lbm_dtype) */
    int32_t device;
    int64_t budget_bytes;   /* device bytes the live solves may hold together */
    int32_t max_slots;      /* 0: no limit */
    int32_t round_steps;    /* steps per round */
    double time_limit;      /* seconds for the whole run, 0: none */
    void *stream;           /* cudaStream_t, or NULL for a private stream */
} lbm_server_config;
typedef struct lbm_request {
    int32_t nx, ny;
    float tau;
    int32_t periodic;
    float body_force[2];
    float wall_velocity[2];
    const uint8_t *flags;   /* host [ny][nx] D2Q9 flags, or NULL (all fluid) */
    int64_t steps;
    double arrival;         /* seconds after the start of the run */
    float *out_rho, *out_ux, *out_uy;  /* host [ny][nx] results, each may be NULL */
} lbm_request;
typedef struct lbm_request_result {
    double admitted, finished;  /* seconds after the start of the run */
    int32_t status;
    int32_t slot;
} lbm_request_result;
typedef struct lbm_server_stats {
    double makespan;        /* seconds from the start to the last completion */
    double cell_updates;    /* sum over requests of cells * steps */
    int64_t rounds;
    int64_t peak_bytes;
    int32_t peak_slots;
    int32_t rejected;
    double round_seconds;   /* device time of the rounds' launch sequences (CUDA events) */
    int32_t tile_shape[3];  /* the batch's final tile shape: cells per thread, block width, rows */
    int32_t tunings;        /* times the batch tuned its tile shape during the run */
} lbm_server_stats;
LBM_API void lbm_server_config_init(lbm_server_config *cfg);
LBM_API lbm_status lbm_server_create(const lbm_server_config *cfg, lbm_server **out);
LBM_API lbm_status lbm_server_destroy(lbm_server *s);
LBM_API const char *lbm_server_last_error(const lbm_server *s);
LBM_API lbm_status lbm_server_run(lbm_server *s, const lbm_request *reqs, int64_t n, lbm_request_result *results,
                                  lbm_server_stats *stats);

/* ---------------------------------------------------------------- allocation-free reduction */
/* No counterpart in the reference.  Mass and momentum sums (FP64) of a D2Q9 population buffer
 * over the fluid cells, for callers that cannot allocate device memory while they run: an
 * application that gives the solver a fixed, fully accounted device budget (an embedding
 * framework that owns all device memory, a serving loop admitting work against a memory budget),
 * or a loop with a latency bound, where cudaMalloc / cudaFree would synchronise the device.
 * The call allocates nothing: every buffer is the caller's, in device memory of the current
 * device, and the per-block partial sums go to a fixed array that the library keeps in device
 * memory (a static array of LBM_NOALLOC_MAX_ROWS / 4 blocks, 192 KiB, held on every GPU that loads
 * the library until the process exits).
 *   dev_populations  unshifted populations, dev_populations[q][ny][row_pitch] (float for LBM_F32,
 *                    double for LBM_F64), q in the D2Q9 order of this header
 *   dev_flags        D2Q9 flags [ny][nx]; only LBM_FLUID cells are summed
 *   dev_out          3 doubles: mass, momentum x, momentum y (written on `stream`)
 *   stream           cudaStream_t (NULL: the legacy default stream)
 * ny above LBM_NOALLOC_MAX_ROWS is rejected with LBM_ERR_INVALID.  The first call on a device looks
 * up the array's device address (with that device current); make that first call before any stream
 * capture.  All calls share the one array: calls whose work overlaps on the GPU race with each
 * other; calls in one stream, or otherwise ordered, do not. */
#define LBM_NOALLOC_MAX_ROWS 32768
LBM_API lbm_status lbm_d2q9_conservation_noalloc(const void *dev_populations, int32_t dtype,
                                                 const uint8_t *dev_flags, int32_t nx, int32_t ny,
                                                 int64_t row_pitch, double *dev_out, void *stream);

/* ---------------------------------------------------------------- seeded geometry generators */
/* Channel of nx x ny: walls on rows 0 and ny-1, ndisks non-overlapping disks (x-periodic
 * distance), centres uniform in [0,nx) x [0,ny), radius uniform in [rmin, rmax]; a cell is
 * solid when its centre (x+0.5, y+0.5) lies inside a disk.  Returns the disks placed as
 * (cx, cy, r) triples in host_disks (may be NULL, else room for 3*ndisks floats). */
LBM_API lbm_status lbm_gen_channel(int32_t nx, int32_t ny, int32_t ndisks, float rmin, float rmax,
                                   uint64_t seed, uint8_t *host_flags, float *host_disks);
/* Lid-driven cavity: moving lid on row ny-1, walls on row 0 and columns 0 and nx-1. */
LBM_API lbm_status lbm_gen_cavity(int32_t nx, int32_t ny, uint8_t *host_flags);
/* Random disks (radius in [rmin, rmax], overlap allowed) added until at least solid_fraction of
 * the cells are solid; existing flags are kept.  Returns the achieved fraction. */
LBM_API lbm_status lbm_gen_disks_fraction(int32_t nx, int32_t ny, float solid_fraction, float rmin,
                                          float rmax, uint64_t seed, uint8_t *host_flags,
                                          float *achieved);

/* ---------------------------------------------------------------- mesh front end (D3Q27_REF)
 * The reference derives the D3Q27_REF cell flags and reflection tables from a closed triangle
 * mesh with CGAL (Model.cpp, Geometry.cpp, Lattice.cpp:228-477).  These calls restate that
 * pipeline on the host; they need no GPU and touch no context.  Lattice index z + Z*(y + Y*x),
 * cell positions spacing * (x, y, z) in float, as the reference. */
typedef struct lbm_mesh lbm_mesh;

typedef struct lbm_mesh_info {
    int64_t vertices;
    int64_t faces;
    int32_t triangle_mesh;   /* every face has 3 vertices */
    int32_t closed;          /* no border edge: Model::isModelClosed (Model.cpp:46-49) */
    int32_t valid;           /* triangle mesh and closed: !Model::checkError() (Model.h) */
    int32_t reserved;
    float bbox_min[3];       /* Model::bounding_box (Model.cpp:70-73) */
    float bbox_max[3];
} lbm_mesh_info;

/* Wavefront OBJ, 'v' and 'f' records (f: 1-based or negative indices, "i/t/n" forms; other
 * records and '#' comments ignored).  Replaces Model::importModel (Model.cpp:22-44); a missing
 * file is an error here (the reference keeps an empty model). */
LBM_API lbm_status lbm_mesh_load_obj(const char *path, lbm_mesh **out);
/* The same from arrays: vertices[3*nv]; face k has face_sizes[k] >= 3 vertices, listed 0-based
 * one face after another in face_indices. */
LBM_API lbm_status lbm_mesh_create(const float *vertices, int64_t nv, const int32_t *face_sizes,
                                   int64_t nf, const int32_t *face_indices, lbm_mesh **out);
LBM_API void lbm_mesh_destroy(lbm_mesh *m);
LBM_API lbm_status lbm_mesh_get_info(const lbm_mesh *m, lbm_mesh_info *out);
/* Model::isPointInsideModel (Model.cpp:51-63): *inside = 1 inside or on the surface, 0 outside
 * or when the mesh is not a closed triangle mesh. */
LBM_API lbm_status lbm_mesh_point_inside(const lbm_mesh *m, const float point[3], int32_t *inside);
/* Model::reflectionVector (Model.cpp:75-91): (p1 - p2) / |p1 - p2| rotated by pi about the normal
 * of the first face hit by the ray from p1 through p2; (0, 0, 0) when the ray hits nothing. */
LBM_API lbm_status lbm_mesh_reflection_vector(const lbm_mesh *m, const float p1[3], const float p2[3],
                                              float out[3]);
/* rotateVectorAroundAxis (Geometry.cpp:22-42): quaternion rotation of v about axis by angle. */
LBM_API void lbm_rotate_vector(const float axis[3], const float v[3], float angle, float out[3]);
/* Lattice::distributeVector (Lattice.cpp:262-321): the 27 directions q ranked by
 * 2 - |v - c_q / |c_q||, highest first, equal scores by the larger q first. */
LBM_API void lbm_distribute_vector(const float v[3], float score_out[27], int32_t dir_out[27]);
/* Lattice::insertModel (Lattice.cpp:228-260): sets LBM_INTERNAL on the cells whose position is
 * inside the mesh and clears it on the others; other flag bits are kept.  A mesh whose bounding
 * box leaves [0, X*spacing] x [0, Y*spacing] x [0, Z*spacing] changes nothing (*applied = 0), as
 * in the reference. */
LBM_API lbm_status lbm_mesh_rasterize(const lbm_mesh *m, int32_t X, int32_t Y, int32_t Z, float spacing,
                                      uint8_t *host_flags, int32_t *applied);
/* Lattice::preProcessModel (Lattice.cpp:323-426): reflection tables for the LBM_INTERNAL cells
 * next to non-internal cells, in the reference's cell order, ready for lbm_set_reflection_tables.
 * With host_cells and host_records NULL only *count is set.  Otherwise capacity must be >=
 * *count; host_cells[i] / host_records[i] (struct ReflectionValues) are written and LBM_REFLECTED
 * is set on those cells.  The reference reads the neighbour in a chosen direction by its linear
 * index without a range check; an index outside the lattice counts as not internal here. */
LBM_API lbm_status lbm_mesh_reflection_tables(const lbm_mesh *m, int32_t X, int32_t Y, int32_t Z,
                                              float spacing, uint8_t *host_flags, int64_t capacity,
                                              int32_t *host_cells, void *host_records, int64_t *count);

#ifdef __cplusplus
}
#endif
#endif /* LBM_CAPI_H */
