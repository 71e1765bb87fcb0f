// D2Q9 update of 16-bit storage with the source rows staged in shared memory by bulk asynchronous
// copies (cp.async.bulk global -> shared, completion counted in bytes on an mbarrier).
//
// Why: the register-blocked vector kernel (d2q9_vec.cuh) holds its loads in flight in registers,
// so the bytes in flight per SM are bounded by registers x resident warps; for 16-bit storage the
// arithmetic per byte is twice that of FP32 and the warps spend too little of their time with
// loads outstanding to cover the HBM latency.  Here one thread of a block issues the copies for
// several rows ahead into a ring of shared-memory slots, independently of the warps that compute.
//
// Block: warp 0 is the producer, warps 1..NC consume.  A task is one row y of a strip of W = NC *
// 32 * V = 512 cells (the library runs V = 4 cells per consumer lane, NC = 4 consumer warps); blocks are
// persistent and take tasks b, b + gridDim.x, ... (in the opposite order with `reverse`).  For a task
// the producer's lane 0 copies into a slot of a ring of K slots the nine plane segments that row y
// pulls - plane q from row y - c_y(q), x0 - 8 .. x0 + W + 8 (the halo keeps every copy 16-byte
// aligned and a multiple of 16 bytes) - and the row's link words, so every population is read from
// HBM once.  In a row periodic in x, lane 1 reads the wrapped columns (x = nx - 1 for the first
// strip, x = 0 for the strip holding the last column) into a small per-slot area with plain loads.
// Bounce-back takes the cells' own populations 1 and 3 from the slot (plane rows of row y) and
// the others from global memory; solid cells are not written.
//
// Per cell the inputs are those of gather() (d2q9_core.cuh) and the update is finish_row()
// (d2q9_vec.cuh), so the results are bit-identical to the other D2Q9 kernels.  Plane elements that
// are not copied (x outside [0, pitch), rows outside [0, ny) when y is not periodic) are stale and
// are only ever read for populations that a link word replaces, or by cells in the row padding,
// whose results are not stored.
//
// Slot protocol, positions counted over the tasks of a block: position p lives in slot p % K;
// full[s] completes when lane 0's expect-tx arrival (and, periodic in x, lane 1's arrival) have
// come and all copied bytes have landed; empty[s] completes when all NC consumer warps have
// released the position after updating its row.  Lanes 0 and 1 refill a slot only once its previous
// position has been released, so the producer runs up to K - 1 rows ahead of the consumers.
//
// Every wait is bounded (wait_ns of wall time, 1 s unless the host sets another limit, or an abort
// raised by another warp of the block): on a timeout the block sets PIPE_TIMEOUT in *status, the
// consumers stop, and lane 0 stops issuing and waits (bounded) for the copies it has issued before
// the block exits.  For testing that path the host can name a task whose copies lane 0 leaves out
// (skip_task >= 0): the consumers' wait for that slot runs out, nothing faults and nothing hangs.
#pragma once

#include "d2q9_vec.cuh"

namespace lbm {
namespace d2q9 {
namespace bulk {

constexpr int W = 512;                 // cells per strip
// consumer warps and block size for V cells per consumer thread
template <int V>
constexpr int consumers() {
    return W / (32 * V);
}
template <int V>
constexpr int threads() {
    return 32 * (consumers<V>() + 1);
}
constexpr int SEG = W + 16;            // staged elements per plane row: x0 - 8 .. x0 + W + 8
constexpr int LINKS = 9 * SEG;         // element offset of the link words in a slot
constexpr int WRAP = 9 * SEG + W;      // wrapped columns: populations 1, 5, 8 at x = nx - 1 of rows y,
                                       // y - 1, y + 1, then populations 3, 6, 7 at x = 0 of those rows
constexpr int SLOT = 9 * SEG + W + 8;  // 16-bit elements per slot
constexpr unsigned PIPE_TIMEOUT = 1u;  // status bit: a bounded wait gave up
static_assert((SLOT * 2) % 16 == 0 && (SEG * 2) % 16 == 0, "slot geometry keeps 16-byte alignment");

// ring of K slots, then K full and K empty barriers, then the abort word
template <int K>
constexpr size_t smem_bytes() {
    return (size_t)K * SLOT * 2 + 2 * K * sizeof(unsigned long long) + 16;
}

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *b, unsigned parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(saddr(b)), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for the phase of parity `parity` of barrier b: false after limit_ns or, when abort is not
// null, once another warp has raised it.
__device__ __forceinline__ bool wait(unsigned long long *b, unsigned parity, const volatile int *abort,
                                     unsigned long long limit_ns) {
    if (mbar_try_wait(b, parity)) return true;
    const unsigned long long t0 = now_ns();
    for (;;) {
        if (mbar_try_wait(b, parity)) return true;
        if (abort && *abort) return false;
        if (now_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void bulk_copy(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     saddr(dst)),
                 "l"(src), "r"(bytes), "r"(saddr(bar))
                 : "memory");
}

// rows y - 1 and y + 1 of row y, wrapped (periodic in y) or clamped
__device__ __forceinline__ void neighbours(int y, int ny, int periodic, int &ym, int &yp) {
    ym = y - 1;
    yp = y + 1;
    if (ym < 0) ym = (periodic & 2) ? ny - 1 : 0;
    if (yp >= ny) yp = (periodic & 2) ? 0 : ny - 1;
}

// task i of nstrips * ny: (strip start, row); adjacent tasks are adjacent strips of a row
__device__ __forceinline__ void task_of(int i, int ntasks, int nstrips, int reverse, int &x0, int &y) {
    if (reverse) i = ntasks - 1 - i;
    y = i / nstrips;
    x0 = (i - y * nstrips) * W;
}

// Lane 0: copy the plane segments and link words row y of the strip at x0 pulls into `slot`, after
// announcing the bytes to expect on `full`.  A plane whose source row lies outside a domain that is
// not periodic in y is not copied.
template <class S>
__device__ __forceinline__ void stage_task(uint16_t *slot, unsigned long long *full, const S *__restrict__ src,
                                           const uint16_t *__restrict__ links, int y, int x0, int ny, int pitch,
                                           int plane, int periodic) {
    const int gx0 = max(x0 - 8, 0), gx1 = min(x0 + W + 8, pitch);
    const int lx1 = min(x0 + W, pitch);
    const unsigned pbytes = (unsigned)(gx1 - gx0) * 2u, lbytes = (unsigned)(lx1 - x0) * 2u;
    // source rows of the three plane groups (c_y = 0: q 0, 1, 3; c_y = +1: q 2, 5, 6; c_y = -1: q 4, 7, 8)
    const bool below = y > 0 || (periodic & 2), above = y < ny - 1 || (periodic & 2);
    const int ym = y > 0 ? y - 1 : ny - 1, yp = y < ny - 1 ? y + 1 : 0;
    mbar_arrive_expect_tx(full, (3u + (below ? 3u : 0u) + (above ? 3u : 0u)) * pbytes + lbytes);
    uint16_t *dst = slot + (gx0 - (x0 - 8));
    const S *g = src + gx0;
    const int64_t r0 = (int64_t)y * pitch, rm = (int64_t)ym * pitch, rp = (int64_t)yp * pitch;
    bulk_copy(dst + 0 * SEG, g + 0 * (int64_t)plane + r0, pbytes, full);
    bulk_copy(dst + 1 * SEG, g + 1 * (int64_t)plane + r0, pbytes, full);
    bulk_copy(dst + 3 * SEG, g + 3 * (int64_t)plane + r0, pbytes, full);
    if (below) {
        bulk_copy(dst + 2 * SEG, g + 2 * (int64_t)plane + rm, pbytes, full);
        bulk_copy(dst + 5 * SEG, g + 5 * (int64_t)plane + rm, pbytes, full);
        bulk_copy(dst + 6 * SEG, g + 6 * (int64_t)plane + rm, pbytes, full);
    }
    if (above) {
        bulk_copy(dst + 4 * SEG, g + 4 * (int64_t)plane + rp, pbytes, full);
        bulk_copy(dst + 7 * SEG, g + 7 * (int64_t)plane + rp, pbytes, full);
        bulk_copy(dst + 8 * SEG, g + 8 * (int64_t)plane + rp, pbytes, full);
    }
    bulk_copy(slot + LINKS, links + r0 + x0, lbytes, full);
}

// Lane 1, periodic in x: the wrapped columns of row y that the strip at x0 needs, then its arrival
template <class S>
__device__ __forceinline__ void stage_wrap(uint16_t *slot, unsigned long long *full, const S *__restrict__ src, int y,
                                           int x0, int nx, int ny, int pitch, int plane, int periodic) {
    int ym, yp;
    neighbours(y, ny, periodic, ym, yp);
    const S *__restrict__ rows[3] = {src + (int64_t)y * pitch, src + (int64_t)ym * pitch, src + (int64_t)yp * pitch};
    S *wr = reinterpret_cast<S *>(slot + WRAP);
    if (x0 == 0) {
        wr[0] = __ldg(rows[0] + 1 * (int64_t)plane + nx - 1);
        wr[1] = __ldg(rows[1] + 5 * (int64_t)plane + nx - 1);
        wr[2] = __ldg(rows[2] + 8 * (int64_t)plane + nx - 1);
    }
    if (nx - 1 >= x0 && nx - 1 < x0 + W) {
        wr[3] = __ldg(rows[0] + 3 * (int64_t)plane);
        wr[4] = __ldg(rows[1] + 6 * (int64_t)plane);
        wr[5] = __ldg(rows[2] + 7 * (int64_t)plane);
    }
    mbar_arrive(full);  // release: the writes above are visible to the consumers' acquiring wait
}

// V consecutive 16-bit elements of shared memory as one access (aligned to 2 V bytes)
template <int V>
__device__ __forceinline__ typename RawPack<2 * V>::T ldsv(const uint16_t *p) {
    return *reinterpret_cast<const typename RawPack<2 * V>::T *>(p);
}

template <class S>
__device__ __forceinline__ S raw_s(uint16_t v) {
    S s;
    memcpy(&s, &v, sizeof(s));
    return s;
}

// One row of the consumer thread t (0 .. W / V - 1): its vector x0 .. x0 + V - 1 of row y, from slot sl.
template <class S, int V, bool FORCE>
__device__ __forceinline__ void update(const uint16_t *sl, const S *__restrict__ src, S *__restrict__ dst, int t,
                                       int x0, int y, int nx, int ny, int pitch, int plane, int periodic,
                                       const D2Q9Params &prm) {
    using R = typename Store<S>::R;
    const int lane = threadIdx.x & 31;
    const int lx = 8 + V * t;
    RowLoad<S, V, int> ld;
    ld.q0 = ldsv<V>(sl + 0 * SEG + lx);
    ld.q2 = ldsv<V>(sl + 2 * SEG + lx);
    ld.q4 = ldsv<V>(sl + 4 * SEG + lx);
    ld.a1 = ldsv<V>(sl + 1 * SEG + lx);
    ld.a5 = ldsv<V>(sl + 5 * SEG + lx);
    ld.a8 = ldsv<V>(sl + 8 * SEG + lx);
    ld.b3 = ldsv<V>(sl + 3 * SEG + lx);
    ld.b6 = ldsv<V>(sl + 6 * SEG + lx);
    ld.b7 = ldsv<V>(sl + 7 * SEG + lx);
    ld.links = ldsv<V>(sl + LINKS + V * t);
    ld.r0 = y * pitch;
    ld.xa = x0;
    const uint16_t *wr = sl + WRAP;
    if (lane == 0) {
        const bool wrap = x0 == 0 && (periodic & 1);  // x = -1 is the column x = nx - 1
        ld.e[0] = raw_s<S>(wrap ? wr[0] : sl[1 * SEG + lx - 1]);
        ld.e[1] = raw_s<S>(wrap ? wr[1] : sl[5 * SEG + lx - 1]);
        ld.e[2] = raw_s<S>(wrap ? wr[2] : sl[8 * SEG + lx - 1]);
    } else if (lane == 31) {
        ld.e[0] = raw_s<S>(sl[3 * SEG + lx + V]);
        ld.e[1] = raw_s<S>(sl[6 * SEG + lx + V]);
        ld.e[2] = raw_s<S>(sl[7 * SEG + lx + V]);
    }
    ld.w[0] = raw_s<S>(wr[3]);  // used by the vector holding the last column of a periodic row only
    ld.w[1] = raw_s<S>(wr[4]);
    ld.w[2] = raw_s<S>(wr[5]);
    // own populations of row y (raw): planes 0, 1, 3 are staged from row y, the others are read
    // from global memory at the clamped vector (a vector beyond the row stores nothing)
    using T = typename RawPack<2 * V>::T;
    const S *mine = src + (int64_t)y * pitch + min(x0, pitch - V);
    auto own = [&](int q) -> T {
        if (q == 0 || q == 1 || q == 3) return ldsv<V>(sl + q * SEG + lx);
        return __ldg(reinterpret_cast<const T *>(mine + (int64_t)q * plane));
    };
    finish_row<S, V, FORCE, int, 0>(ld, own, dst, x0, nx, plane, periodic, prm, 0, ld.e, ld.e, lane == 0, lane == 31,
                                    true);
}

template <class S, int V, bool FORCE, int K>
__device__ __forceinline__ void pipeline(unsigned char *smem, const S *__restrict__ src, S *__restrict__ dst,
                                         const uint16_t *__restrict__ links, int nx, int ny, int pitch, int plane,
                                         int periodic, const D2Q9Params &prm, int reverse, unsigned *status,
                                         unsigned long long wait_ns, int skip_task) {
    static_assert(sizeof(S) == 2, "the bulk-copy pipeline is for 16-bit storage");
    static_assert(K >= 2, "a ring of at least two slots");
    uint16_t *ring = reinterpret_cast<uint16_t *>(smem);
    unsigned long long *full = reinterpret_cast<unsigned long long *>(smem + (size_t)K * SLOT * 2);
    unsigned long long *empty = full + K;
    volatile int *abort = reinterpret_cast<volatile int *>(empty + K);
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    const bool wrap_x = periodic & 1;
    if (threadIdx.x == 0) {
        for (int s = 0; s < K; ++s) {
            mbar_init(&full[s], wrap_x ? 2 : 1);
            mbar_init(&empty[s], consumers<V>());
        }
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    const int nstrips = (pitch + W - 1) / W;
    const int ntasks = nstrips * ny;

    if (warp == 0) {  // producer: lane 0 copies, lane 1 reads the wrapped columns
        if (lane > 1 || (lane == 1 && !wrap_x)) return;
        unsigned pos = 0;
        bool ok = true;
        int skipped = -1;  // position whose copies were left out (skip_task)
        for (int i = blockIdx.x; i < ntasks; i += gridDim.x, ++pos) {
            const unsigned s = pos % K;
            if (pos >= (unsigned)K && !wait(&empty[s], ((pos / K) - 1) & 1u, abort, wait_ns)) {
                ok = false;
                break;
            }
            int x0, y;
            task_of(i, ntasks, nstrips, reverse, x0, y);
            uint16_t *slot = ring + (size_t)s * SLOT;
            if (lane == 0) {
                if (i == skip_task)
                    skipped = (int)pos;  // no copy and no arrival: the consumers' wait runs out
                else
                    stage_task<S>(slot, &full[s], src, links, y, x0, ny, pitch, plane, periodic);
            } else {
                stage_wrap<S>(slot, &full[s], src, y, x0, nx, ny, pitch, plane, periodic);
            }
        }
        if (!ok) {
            *abort = 1;
            atomicOr(status, PIPE_TIMEOUT);
            // the copies lane 0 issued land before the block's shared memory goes away
            if (lane == 0)
                for (unsigned q = pos > (unsigned)K ? pos - K : 0u; q < pos; ++q)
                    if ((int)q != skipped) wait(&full[q % K], (q / K) & 1u, nullptr, wait_ns);
        }
        return;
    }

    // consumers
    const int t = (warp - 1) * 32 + lane;
    unsigned pos = 0;
    for (int i = blockIdx.x; i < ntasks; i += gridDim.x, ++pos) {
        const unsigned s = pos % K;
        if (!__all_sync(0xffffffffu, wait(&full[s], (pos / K) & 1u, abort, wait_ns))) {
            if (lane == 0) {
                *abort = 1;
                atomicOr(status, PIPE_TIMEOUT);
            }
            return;
        }
        int x0, y;
        task_of(i, ntasks, nstrips, reverse, x0, y);
        update<S, V, FORCE>(ring + (size_t)s * SLOT, src, dst, t, x0 + V * t, y, nx, ny, pitch, plane, periodic, prm);
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    }
}

}  // namespace bulk
}  // namespace d2q9
}  // namespace lbm
