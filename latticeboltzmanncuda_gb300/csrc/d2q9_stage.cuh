// Row-sweep D2Q9 update with the source populations staged through shared memory (16-bit storage).
//
// A block of THREADS threads owns a strip of W = 2 * THREADS consecutive cells and a run of rows
// [ya, yb).  It keeps a ring of NSLOT row slots in shared memory; a slot holds the nine population
// planes of one source row from x0 - 8 to x0 + W + 8 (the 8-element halo keeps every copy a whole,
// aligned 16-byte chunk).  Rows are copied in with cp.async up to NSLOT - 3 rows ahead of the row
// being computed, so the bytes in flight per SM are set by the ring depth rather than by the
// registers each thread holds -- the limit of the register-blocked kernel for 16-bit storage, whose
// 8-cell vectors need ~128 registers per thread.  Every source row is read from HBM once per strip
// (plus one row above and below the run); each output row is written with 4-byte stores, two cells
// per thread.
//
// Per cell the inputs are exactly those of gather() (d2q9_core.cuh): pulled values from the staged
// rows, the periodic wrap of the first and last column read from global memory, bounce-back and
// moving-wall values from the cell's own staged row, solid cells copying their own populations; the
// collision is the shared collide(), so results are bit-identical to the other D2Q9 kernels.
//
// Synchronisation: one __syncthreads() per row, executed by every thread of the block (no thread
// leaves the loop early); cp.async.wait_group waits only for the calling thread's own copies.
#pragma once

#include "d2q9_core.cuh"

namespace lbm {
namespace d2q9 {
namespace stage {

constexpr int THREADS = 128;
constexpr int W = 2 * THREADS;     // cells per strip
constexpr int SEG = W + 16;        // staged elements per plane row: x0 - 8 .. x0 + W + 8
constexpr int CHUNKS = SEG / 8;    // 16-byte chunks per plane row (16-bit elements)
constexpr int NSLOT = 8;           // ring depth: rows y-1, y, y+1 and NSLOT - 3 rows ahead
static_assert(SEG % 8 == 0 && (NSLOT & (NSLOT - 1)) == 0, "stage geometry");

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Ring storage of one block: [slot][plane][element], 16-byte aligned rows.
template <class S>
struct Ring {
    alignas(16) S v[NSLOT][9][SEG];
};

// Copy source row `row` (before wrapping) into ring slot `slot`; rows outside [0, ny) wrap when the
// lattice is periodic in y and are zero otherwise (their values are never used: the cells next to a
// non-periodic edge bounce those populations back).  Chunks outside [0, pitch) are zero.
template <class S>
__device__ __forceinline__ void load_row(Ring<S> &ring, int slot, const S *__restrict__ src, int row, int x0, int ny,
                                         int pitch, int plane, int periodic) {
    bool valid = true;
    if (row < 0 || row >= ny) {
        if (periodic & 2)
            row = row < 0 ? row + ny : row - ny;
        else
            valid = false;
    }
    for (int i = (int)threadIdx.x; i < 9 * CHUNKS; i += THREADS) {
        const int q = i / CHUNKS, j = i - q * CHUNKS;
        const int gx = x0 - 8 + 8 * j;
        S *d = &ring.v[slot][q][8 * j];
        if (valid && gx >= 0 && gx + 8 <= pitch)
            cp_async16(d, src + (int64_t)q * plane + (int64_t)row * pitch + gx);
        else
            *reinterpret_cast<uint4 *>(d) = make_uint4(0u, 0u, 0u, 0u);
    }
}

// one cell: sp / sc / sn are the slots of rows y-1 / y / y+1, lx the cell's index in a slot row
template <class S, bool FORCE>
__device__ __forceinline__ void cell(const Ring<S> &ring, int sp, int sc, int sn, int lx, uint32_t L,
                                     const S *__restrict__ src, int x, int y, int nx, int ny, int pitch, int plane,
                                     int periodic, const D2Q9Params &prm, S out[9]) {
    using R = typename Store<S>::R;
    if (L == LINK_SOLID) {
#pragma unroll
        for (int q = 0; q < 9; ++q) out[q] = ring.v[sc][q][lx];
        return;
    }
    R h[9];
    h[0] = Store<S>::to(ring.v[sc][0][lx]);
    h[1] = Store<S>::to(ring.v[sc][1][lx - 1]);
    h[2] = Store<S>::to(ring.v[sp][2][lx]);
    h[3] = Store<S>::to(ring.v[sc][3][lx + 1]);
    h[4] = Store<S>::to(ring.v[sn][4][lx]);
    h[5] = Store<S>::to(ring.v[sp][5][lx - 1]);
    h[6] = Store<S>::to(ring.v[sp][6][lx + 1]);
    h[7] = Store<S>::to(ring.v[sn][7][lx + 1]);
    h[8] = Store<S>::to(ring.v[sn][8][lx - 1]);
    if ((periodic & 1) && (x == 0 || x == nx - 1)) {
        // the wrapped column lies outside the strip: read it as gather() does
        int ym = y - 1, yp = y + 1;
        if (ym < 0) ym = (periodic & 2) ? ny - 1 : 0;
        if (yp >= ny) yp = (periodic & 2) ? 0 : ny - 1;
        const int64_t r0 = (int64_t)y * pitch, rm = (int64_t)ym * pitch, rp = (int64_t)yp * pitch;
        if (x == 0) {
            const int xm = nx - 1;
            h[1] = ldh<S>(src + 1 * (int64_t)plane + r0 + xm);
            h[5] = ldh<S>(src + 5 * (int64_t)plane + rm + xm);
            h[8] = ldh<S>(src + 8 * (int64_t)plane + rp + xm);
        }
        if (x == nx - 1) {
            h[3] = ldh<S>(src + 3 * (int64_t)plane + r0);
            h[6] = ldh<S>(src + 6 * (int64_t)plane + rm);
            h[7] = ldh<S>(src + 7 * (int64_t)plane + rp);
        }
    }
    if (L) {
        const Vec2<R> uw = wall_u<R>(prm);
#pragma unroll
        for (int q = 1; q < 9; ++q) {
            if (L & (1u << (q - 1))) {
                R v = Store<S>::to(ring.v[sc][opp(q)][lx]);
                if (L & (1u << (q + 7))) v = add_(v, wall_term<S, R>(q, uw));
                h[q] = v;
            }
        }
    }
    collide<S, R, FORCE>(h, omega<R>(prm), force<R>(prm));
#pragma unroll
    for (int q = 0; q < 9; ++q) out[q] = Store<S>::from(h[q]);
}

// Advance rows [ya, yb) of the strip starting at x0 (a multiple of W) by one step.
template <class S, bool FORCE>
__device__ __forceinline__ void sweep(Ring<S> &ring, const S *__restrict__ src, S *__restrict__ dst,
                                      const uint16_t *__restrict__ links, int x0, int ya, int yb, int nx, int ny,
                                      int pitch, int plane, int periodic, const D2Q9Params &prm) {
    static_assert(sizeof(S) == 2, "the staged sweep is for 16-bit storage");
    const int nrows = yb - ya;      // uniform across the block
    const int npos = nrows + 2;     // staged rows ya-1 .. yb
    // prologue: positions 0 .. NSLOT-2 (one commit group each, empty past the last row)
#pragma unroll 1
    for (int p = 0; p < NSLOT - 1; ++p) {
        if (p < npos) load_row<S>(ring, p & (NSLOT - 1), src, ya - 1 + p, x0, ny, pitch, plane, periodic);
        cp_async_commit();
    }
    const int tx = (int)threadIdx.x;
    const int xa = x0 + 2 * tx;
#pragma unroll 1
    for (int k = 0; k < nrows; ++k) {
        // positions <= k+2 have landed once at most NSLOT-4 of this thread's groups are pending
        cp_async_wait<NSLOT - 4>();
        __syncthreads();
        {
            const int p = k + NSLOT - 1;  // refills the slot of position k-1, no longer read
            if (p < npos) load_row<S>(ring, p & (NSLOT - 1), src, ya - 1 + p, x0, ny, pitch, plane, periodic);
            cp_async_commit();
        }
        const int y = ya + k;
        const int sp = k & (NSLOT - 1), sc = (k + 1) & (NSLOT - 1), sn = (k + 2) & (NSLOT - 1);
        if (xa < nx) {
            const int64_t c = (int64_t)y * pitch + xa;
            const uint32_t L2 = __ldg(reinterpret_cast<const uint32_t *>(links + c));
            S o0[9], o1[9];
            cell<S, FORCE>(ring, sp, sc, sn, 2 * tx + 8, L2 & 0xffffu, src, xa, y, nx, ny, pitch, plane, periodic, prm, o0);
            // the second cell may lie in the row padding (odd nx): computed, stored there, never read
            cell<S, FORCE>(ring, sp, sc, sn, 2 * tx + 9, L2 >> 16, src, xa + 1, y, nx, ny, pitch, plane, periodic, prm, o1);
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                S pair[2] = {o0[q], o1[q]};
                uint32_t raw;
                memcpy(&raw, pair, sizeof(raw));
                *reinterpret_cast<uint32_t *>(dst + (int64_t)q * plane + c) = raw;
            }
        }
    }
    cp_async_wait<0>();  // no copy outlives the block
}

}  // namespace stage
}  // namespace d2q9
}  // namespace lbm
