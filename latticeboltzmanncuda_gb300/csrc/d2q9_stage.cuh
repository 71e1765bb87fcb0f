// Row-sweep D2Q9 update with the source rows staged through shared memory (16-bit storage).
//
// A block of THREADS = 128 threads owns a strip of W = 512 consecutive cells (4 per thread) and a
// run of rows [ya, yb).  It keeps a ring of NSLOT row slots in shared memory; a slot holds the nine
// population planes of one source row from x0 - 8 to x0 + W + 8 (the 8-element halo keeps every
// copy a whole, aligned 16-byte chunk) and the row's link words.  Rows are copied in with cp.async
// up to NSLOT - 3 rows ahead of the row being computed, so the bytes in flight per SM are set by
// the ring rather than by the registers a thread holds (the limit of the register-blocked kernel,
// whose 8-cell vectors of 16-bit values need ~128 registers per thread).  Every source row is read
// from HBM once per strip (plus one row above and below the run); output rows are written with
// 8-byte stores, four cells per thread.
//
// Copies: thread j < CHUNKS copies chunk j of all nine plane rows, threads THREADS - LCHUNKS ..
// THREADS - 1 one chunk of link words each.  Chunks outside [0, pitch) and rows outside [0, ny)
// (not periodic in y) are not copied: those slot elements are only ever read for populations that
// the cell's link word replaces by bounce-back, or by the periodic-column patch below, or by cells
// in the row padding whose results are never read.
//
// Per cell the inputs are exactly those of gather() (d2q9_core.cuh): pulled values from the staged
// rows, the periodic wrap of the first and last column read from global memory, bounce-back and
// moving-wall values from the cell's own row, solid cells copying their own populations; the
// collision is the shared collide(), so results are bit-identical to the other D2Q9 kernels.
//
// Synchronisation: one __syncthreads() per row, reached by every thread of the block (no thread
// leaves the loop); cp.async.wait_group waits only for the calling thread's own copies, which
// always complete.
#pragma once

#include "d2q9_core.cuh"

namespace lbm {
namespace d2q9 {
namespace stage {

constexpr int THREADS = 128;
constexpr int CPT = 4;               // cells per thread
constexpr int W = THREADS * CPT;     // cells per strip
constexpr int SEG = W + 16;          // staged elements per plane row: x0 - 8 .. x0 + W + 8
constexpr int CHUNKS = SEG / 8;      // 16-byte chunks per plane row
constexpr int LCHUNKS = W / 8;       // 16-byte chunks of link words per row
constexpr int LINKS = 9 * SEG;       // element offset of the link words in a slot
constexpr int SLOT = 9 * SEG + W;    // 16-bit elements per slot
static_assert(CHUNKS <= THREADS && LCHUNKS <= THREADS && (SLOT * 2) % 16 == 0, "stage geometry");

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Ring of NSLOT slots, [slot][SLOT] 16-bit elements (dynamic shared memory, 16-byte aligned).
template <int NSLOT>
constexpr size_t ring_bytes() {
    return (size_t)NSLOT * SLOT * 2;
}

// Issue the copies of source row `row` (before wrapping) into `slot`.
template <class S>
__device__ __forceinline__ void load_row(uint16_t *slot, const S *__restrict__ src, const uint16_t *__restrict__ links,
                                         int row, int x0, int ny, int pitch, int plane, int periodic) {
    if (row < 0 || row >= ny) {
        if (!(periodic & 2)) return;
        row = row < 0 ? row + ny : row - ny;
    }
    const int t = (int)threadIdx.x;
    const int64_t roff = (int64_t)row * pitch;
    if (t < CHUNKS) {
        const int gx = x0 - 8 + 8 * t;
        if (gx >= 0 && gx + 8 <= pitch) {
            const S *g = src + roff + gx;
#pragma unroll
            for (int q = 0; q < 9; ++q) cp_async16(slot + q * SEG + 8 * t, g + (int64_t)q * plane);
        }
    }
    const int lt = t - (THREADS - LCHUNKS);
    if (lt >= 0) {
        const int gx = x0 + 8 * lt;
        if (gx + 8 <= pitch) cp_async16(slot + LINKS + 8 * lt, links + roff + gx);
    }
}

// element k (0..3) of four consecutive 16-bit values held in a uint2
__device__ __forceinline__ uint16_t el(uint2 v, int k) {
    const uint32_t w = k < 2 ? v.x : v.y;
    return (uint16_t)((k & 1) ? (w >> 16) : (w & 0xffffu));
}

template <class S>
__device__ __forceinline__ typename Store<S>::R val(uint16_t raw) {
    S s;
    memcpy(&s, &raw, sizeof(s));
    return Store<S>::to(s);
}

__device__ __forceinline__ uint2 lds64(const uint16_t *p) { return *reinterpret_cast<const uint2 *>(p); }

// Advance rows [ya, yb) of the strip starting at x0 (a multiple of W) by one step.
template <class S, bool FORCE, int NSLOT>
__device__ __forceinline__ void sweep(uint16_t *ring, const S *__restrict__ src, S *__restrict__ dst,
                                      const uint16_t *__restrict__ links, int x0, int ya, int yb, int nx, int ny,
                                      int pitch, int plane, int periodic, const D2Q9Params &prm) {
    static_assert(sizeof(S) == 2, "the staged sweep is for 16-bit storage");
    static_assert(NSLOT >= 4 && (NSLOT & (NSLOT - 1)) == 0, "ring depth");
    using R = typename Store<S>::R;
    const int nrows = yb - ya;   // uniform across the block
    const int npos = nrows + 2;  // staged rows ya-1 .. yb
#pragma unroll 1
    for (int p = 0; p < NSLOT - 1; ++p) {
        if (p < npos) load_row<S>(ring + (p & (NSLOT - 1)) * SLOT, src, links, ya - 1 + p, x0, ny, pitch, plane, periodic);
        cp_async_commit();
    }
    const int t = (int)threadIdx.x;
    const int xa = x0 + CPT * t;
    const int lx = 8 + CPT * t;  // first cell's element in a slot row
#pragma unroll 1
    for (int k = 0; k < nrows; ++k) {
        cp_async_wait<NSLOT - 4>();  // positions <= k+2 have landed
        __syncthreads();
        {
            const int p = k + NSLOT - 1;  // refills the slot of position k-1, no longer read
            if (p < npos) load_row<S>(ring + (p & (NSLOT - 1)) * SLOT, src, links, ya - 1 + p, x0, ny, pitch, plane, periodic);
            cp_async_commit();
        }
        if (xa >= nx) continue;
        const int y = ya + k;
        const uint16_t *rp = ring + (k & (NSLOT - 1)) * SLOT;        // row y-1
        const uint16_t *rc = ring + ((k + 1) & (NSLOT - 1)) * SLOT;  // row y
        const uint16_t *rn = ring + ((k + 2) & (NSLOT - 1)) * SLOT;  // row y+1
        // the four cells' pulled values: plane q from row y - cy_q at x - cx_q
        const uint2 a0 = lds64(rc + 0 * SEG + lx), a2 = lds64(rp + 2 * SEG + lx), a4 = lds64(rn + 4 * SEG + lx);
        const uint2 a1 = lds64(rc + 1 * SEG + lx), a5 = lds64(rp + 5 * SEG + lx), a8 = lds64(rn + 8 * SEG + lx);
        const uint2 a3 = lds64(rc + 3 * SEG + lx), a6 = lds64(rp + 6 * SEG + lx), a7 = lds64(rn + 7 * SEG + lx);
        const uint16_t e1 = rc[1 * SEG + lx - 1], e5 = rp[5 * SEG + lx - 1], e8 = rn[8 * SEG + lx - 1];
        const uint16_t e3 = rc[3 * SEG + lx + 4], e6 = rp[6 * SEG + lx + 4], e7 = rn[7 * SEG + lx + 4];
        const uint2 ll = lds64(rc + LINKS + CPT * t);
        uint32_t out[9][2];
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            const int x = xa + c;
            const uint32_t L = el(ll, c);
            uint16_t o[9];
            if (L == LINK_SOLID) {
                // solid: copy the cell's own populations
#pragma unroll
                for (int q = 0; q < 9; ++q) o[q] = rc[q * SEG + lx + c];
            } else {
                R h[9];
                h[0] = val<S>(el(a0, c));
                h[2] = val<S>(el(a2, c));
                h[4] = val<S>(el(a4, c));
                h[1] = val<S>(c == 0 ? e1 : el(a1, c - 1));
                h[5] = val<S>(c == 0 ? e5 : el(a5, c - 1));
                h[8] = val<S>(c == 0 ? e8 : el(a8, c - 1));
                h[3] = val<S>(c == CPT - 1 ? e3 : el(a3, c + 1));
                h[6] = val<S>(c == CPT - 1 ? e6 : el(a6, c + 1));
                h[7] = val<S>(c == CPT - 1 ? e7 : el(a7, c + 1));
                if ((periodic & 1) && (x == 0 || x == nx - 1)) {
                    // the wrapped column lies outside the strip: read it as gather() does
                    int ym = y - 1, yp = y + 1;
                    if (ym < 0) ym = (periodic & 2) ? ny - 1 : 0;
                    if (yp >= ny) yp = (periodic & 2) ? 0 : ny - 1;
                    const int64_t r0 = (int64_t)y * pitch, rm = (int64_t)ym * pitch, rq = (int64_t)yp * pitch;
                    if (x == 0) {
                        const int xm = nx - 1;
                        h[1] = ldh<S>(src + 1 * (int64_t)plane + r0 + xm);
                        h[5] = ldh<S>(src + 5 * (int64_t)plane + rm + xm);
                        h[8] = ldh<S>(src + 8 * (int64_t)plane + rq + xm);
                    }
                    if (x == nx - 1) {
                        h[3] = ldh<S>(src + 3 * (int64_t)plane + r0);
                        h[6] = ldh<S>(src + 6 * (int64_t)plane + rm);
                        h[7] = ldh<S>(src + 7 * (int64_t)plane + rq);
                    }
                }
                if (L) {
                    const Vec2<R> uw = wall_u<R>(prm);
#pragma unroll
                    for (int q = 1; q < 9; ++q) {
                        if (L & (1u << (q - 1))) {
                            R v = val<S>(rc[opp(q) * SEG + lx + c]);
                            if (L & (1u << (q + 7))) v = add_(v, wall_term<S, R>(q, uw));
                            h[q] = v;
                        }
                    }
                }
                collide<S, R, FORCE>(h, omega<R>(prm), force<R>(prm));
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    const S s = Store<S>::from(h[q]);
                    memcpy(&o[q], &s, sizeof(s));
                }
            }
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                if (c & 1)
                    out[q][c >> 1] |= (uint32_t)o[q] << 16;
                else
                    out[q][c >> 1] = o[q];
            }
        }
        // cells beyond the last column (xa + c >= nx) were computed from padding and land in the
        // row padding, which no cell reads
        const int64_t cofs = (int64_t)y * pitch + xa;
#pragma unroll
        for (int q = 0; q < 9; ++q)
            *reinterpret_cast<uint2 *>(dst + (int64_t)q * plane + cofs) = make_uint2(out[q][0], out[q][1]);
    }
    cp_async_wait<0>();  // no copy outlives the block
}

}  // namespace stage
}  // namespace d2q9
}  // namespace lbm
