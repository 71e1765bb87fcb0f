// Two D2Q9 time steps per launch on a shared-memory tile (temporal blocking).
//
// A block owns an output tile of TX x TY cells.  It loads the source populations of the tile and a
// halo of two cells on every side (the tile grown by 2: what two pull steps reach), computes the
// first step for the tile grown by 1 into a second shared-memory tile, and the second step for the
// tile itself into the destination buffer.  The populations are read from and written to HBM once
// per two updates; the halo's first-step cells are computed by both neighbouring blocks.
//
// Per cell the update is scalar_cell()'s (d2q9_vec.cuh) -- the same pulls, bounce-back and
// moving-wall terms, and the same collision -- and the first step's values are held in the storage
// type, rounded as the one-step kernel stores them, so two steps here are bit-identical to two
// launches of the one-step kernels.  Solid cells are not written (their values are never read:
// a pull from a solid cell is replaced by bounce-back).  Halo cells outside a non-periodic domain
// are loaded from a clamped position; their first-step values are computed from whatever the tile
// holds and never read: a cell at the domain edge replaces every pull from outside by bounce-back.
// Cells go two at a time (adjacent in a row) through the packed FP32 collision, which rounds each
// lane as the scalar one does.
#pragma once

#include "d2q9_core.cuh"

namespace lbm {
namespace d2q9 {
namespace tile2 {

constexpr int THREADS = 256;

template <class S, int TX, int TY>
struct Layout {
    static constexpr int IW = TX + 4, IH = TY + 4;  // the loaded tile: two halo cells each side
    static constexpr int MW = TX + 2, MH = TY + 2;  // the first step's tile: one halo cell
    static constexpr int IN = IW * IH, MN = MW * MH;
    // shared memory: in[9][IH][IW] and mid[9][MH][MW] in the storage type, then the link words of
    // the mid tile
    static constexpr size_t in_bytes = (size_t)9 * IN * sizeof(S);
    static constexpr size_t mid_bytes = (size_t)9 * MN * sizeof(S);
    static constexpr size_t bytes = in_bytes + mid_bytes + (size_t)MN * sizeof(uint16_t);
};

__device__ __forceinline__ int wrap_or_clamp(int g, int n, bool periodic, bool &inside) {
    if (g >= 0 && g < n) return g;
    if (periodic) {
        int r = g % n;
        return r < 0 ? r + n : r;
    }
    inside = false;
    return g < 0 ? 0 : n - 1;
}

// Populations of the cells (ci, cj) and (ci + 1, cj) of a tile T[9][H][W] (row width W, N cells a
// plane) as FP32 pairs: their pulls from (ci - c_x, cj - c_y), replaced by the cell's own opposite
// population where link bit q - 1 is set (plus the moving-wall term where bit q + 7 is).
template <class S, int W, int N>
__device__ __forceinline__ void gather_pair(const S *T, int ci, int cj, uint32_t L0, uint32_t L1, Vec2<float> uw,
                                            float2 h[9]) {
    const int c = cj * W + ci;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const int s = q * N + c - cy(q) * W - cx(q);
        h[q] = make_float2(Store<S>::to(T[s]), Store<S>::to(T[s + 1]));
    }
    if (L0 | L1) {
#pragma unroll
        for (int q = 1; q < 9; ++q) {
            const uint32_t b = 1u << (q - 1), wb = 1u << (q + 7);
            if ((L0 | L1) & b) {
                const int o = opp(q) * N + c;
                if (L0 & b) {
                    float v = Store<S>::to(T[o]);
                    if (L0 & wb) v = add_(v, wall_term<S, float>(q, uw));
                    h[q].x = v;
                }
                if (L1 & b) {
                    float v = Store<S>::to(T[o + 1]);
                    if (L1 & wb) v = add_(v, wall_term<S, float>(q, uw));
                    h[q].y = v;
                }
            }
        }
    }
}

// V consecutive storage elements as one access (2 for the pairs here)
template <class S>
struct PairRaw {
    using T = typename RawPack<2 * sizeof(S)>::T;
};

template <class S, int TX, int TY, bool FORCE>
__device__ __forceinline__ void two_steps(const S *__restrict__ src, S *__restrict__ dst,
                                          const uint16_t *__restrict__ links, int nx, int ny, int pitch,
                                          int plane, int periodic, const D2Q9Params &prm, unsigned char *smem) {
    using Lay = Layout<S, TX, TY>;
    using P = typename PairRaw<S>::T;  // two elements of storage
    static_assert(TX % 2 == 0 && Lay::IW % 2 == 0 && Lay::MW % 2 == 0, "cells go in pairs");
    S *in = reinterpret_cast<S *>(smem);
    S *mid = reinterpret_cast<S *>(smem + Lay::in_bytes);
    uint16_t *lk = reinterpret_cast<uint16_t *>(smem + Lay::in_bytes + Lay::mid_bytes);
    const int x0 = (int)blockIdx.x * TX, y0 = (int)blockIdx.y * TY;
    const bool px = periodic & 1, py = periodic & 2;

    // the source tile with its two-cell halo, a pair of cells at a time (wrapped when periodic,
    // clamped otherwise); a pair that is not two consecutive elements of one row goes one by one
    for (int k = (int)threadIdx.x; k < Lay::IN / 2; k += THREADS) {
        const int j = k / (Lay::IW / 2), i = 2 * (k - j * (Lay::IW / 2));
        bool in0 = true, in1 = true, iny = true;
        const int gx0 = wrap_or_clamp(x0 - 2 + i, nx, px, in0);
        const int gx1 = wrap_or_clamp(x0 - 1 + i, nx, px, in1);
        const int gy = wrap_or_clamp(y0 - 2 + j, ny, py, iny);
        const int g = gy * pitch + gx0;
        const int t = j * Lay::IW + i;
        if (gx1 == gx0 + 1 && (gx0 & 1) == 0) {
#pragma unroll
            for (int q = 0; q < 9; ++q)
                *reinterpret_cast<P *>(in + q * Lay::IN + t) = __ldg(reinterpret_cast<const P *>(src + (size_t)q * plane + g));
        } else {
            const int g1 = gy * pitch + gx1;
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                in[q * Lay::IN + t] = __ldg(src + (size_t)q * plane + g);
                in[q * Lay::IN + t + 1] = __ldg(src + (size_t)q * plane + g1);
            }
        }
    }
    // the link words of the first step's tile; 0xFFFF for a cell outside the domain (only the first
    // step reads it there, and computes that cell from garbage that no output cell reads)
    for (int k = (int)threadIdx.x; k < Lay::MN; k += THREADS) {
        const int j = k / Lay::MW, i = k - j * Lay::MW;
        bool inside = true;
        const int gx = wrap_or_clamp(x0 - 1 + i, nx, px, inside);
        const int gy = wrap_or_clamp(y0 - 1 + j, ny, py, inside);
        lk[k] = inside ? __ldg(links + gy * pitch + gx) : (uint16_t)0xFFFF;
    }
    __syncthreads();

    const float om = omega<float>(prm);
    const Vec2<float> F = force<float>(prm), uw = wall_u<float>(prm);
    // first step, two cells at a time: the tile grown by one cell (mid cell (i, j) is in-tile cell
    // (i + 1, j + 1)).  A cell outside the domain or solid is computed from whatever its tile holds
    // and its result never read.
    for (int k = (int)threadIdx.x; k < Lay::MN / 2; k += THREADS) {
        const int j = k / (Lay::MW / 2), i = 2 * (k - j * (Lay::MW / 2));
        const int m = j * Lay::MW + i;
        const uint32_t L0 = lk[m], L1 = lk[m + 1];
        float2 h[9];
        gather_pair<S, Lay::IW, Lay::IN>(in, i + 1, j + 1, L0 == LINK_SOLID ? 0u : L0, L1 == LINK_SOLID ? 0u : L1,
                                         uw, h);
        collide_t<S, float2, FORCE>(h, om, F);
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const S a = Store<S>::from(h[q].x), b = Store<S>::from(h[q].y);
            mid[q * Lay::MN + m] = a;
            mid[q * Lay::MN + m + 1] = b;
        }
    }
    __syncthreads();

    // second step, two cells at a time: the tile itself (output cell (i, j) is mid cell
    // (i + 1, j + 1)), into dst; solid cells and cells beyond the domain are not written
    for (int k = (int)threadIdx.x; k < TX * TY / 2; k += THREADS) {
        const int j = k / (TX / 2), i = 2 * (k - j * (TX / 2));
        const int x = x0 + i, y = y0 + j;
        if (x >= nx || y >= ny) continue;
        const int m = (j + 1) * Lay::MW + (i + 1);
        const uint32_t L0 = lk[m], L1 = lk[m + 1];
        // (an output cell lies in the domain: its word is its link word, never the outside marker)
        const bool w0 = L0 != LINK_SOLID, w1 = x + 1 < nx && L1 != LINK_SOLID;
        if (!w0 && !w1) continue;
        float2 h[9];
        gather_pair<S, Lay::MW, Lay::MN>(mid, i + 1, j + 1, w0 ? L0 : 0u, w1 ? L1 : 0u, uw, h);
        collide_t<S, float2, FORCE>(h, om, F);
        const int g = y * pitch + x;
        if (w0 && w1) {
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                P raw;
                if constexpr (sizeof(S) == 2) {
                    const typename Pair<S>::P p2 = Pair<S>::from(h[q].x, h[q].y);
                    memcpy(&raw, &p2, sizeof(raw));
                } else {
                    const S e[2] = {Store<S>::from(h[q].x), Store<S>::from(h[q].y)};
                    memcpy(&raw, e, sizeof(raw));
                }
                *reinterpret_cast<P *>(dst + (size_t)q * plane + g) = raw;
            }
        } else {
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                if (w0) dst[(size_t)q * plane + g] = Store<S>::from(h[q].x);
                if (w1) dst[(size_t)q * plane + g + 1] = Store<S>::from(h[q].y);
            }
        }
    }
}

// Persistent form: a block loops over tiles t = blockIdx.x, blockIdx.x + gridDim.x, ... and issues
// the next tile's copies (`cp.async`: the populations and the link words of the loaded tile, two
// aligned elements at a time) into the second of two input buffers before it computes the current
// tile, so the copies overlap the arithmetic.  The link words are taken over the loaded tile (the
// first step's cells are its interior); a cell outside a non-periodic domain carries the link word
// of the clamped position, and like every other first-step cell outside the domain its result is
// never read.
template <class S, int TX, int TY>
struct LayoutP {
    using L = Layout<S, TX, TY>;
    static constexpr size_t in_bytes = L::in_bytes;                             // one input buffer
    static constexpr size_t lk_bytes = (size_t)L::IN * sizeof(uint16_t);        // its link words
    static constexpr size_t buf_bytes = (in_bytes + lk_bytes + 15) / 16 * 16;   // one buffer
    static constexpr size_t bytes = 2 * buf_bytes + L::mid_bytes;
};

template <int BYTES>
__device__ __forceinline__ void copy_async(void *smem_dst, const void *gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(d), "l"(gmem_src), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void copy_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void copy_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <class S, int TX, int TY, int NT>
__device__ __forceinline__ void issue_tile(const S *__restrict__ src, const uint16_t *__restrict__ links, int nx,
                                           int ny, int pitch, int plane, bool px, bool py, int x0, int y0, S *in,
                                           uint16_t *lk) {
    using Lay = Layout<S, TX, TY>;
    using P = typename PairRaw<S>::T;
    for (int k = (int)threadIdx.x; k < Lay::IN / 2; k += NT) {
        const int j = k / (Lay::IW / 2), i = 2 * (k - j * (Lay::IW / 2));
        bool in0 = true, in1 = true, iny = true;
        const int gx0 = wrap_or_clamp(x0 - 2 + i, nx, px, in0);
        const int gx1 = wrap_or_clamp(x0 - 1 + i, nx, px, in1);
        const int gy = wrap_or_clamp(y0 - 2 + j, ny, py, iny);
        const int g = gy * pitch + gx0;
        const int t = j * Lay::IW + i;
        if (gx1 == gx0 + 1 && (gx0 & 1) == 0) {
#pragma unroll
            for (int q = 0; q < 9; ++q) copy_async<sizeof(P)>(in + q * Lay::IN + t, src + (size_t)q * plane + g);
            copy_async<4>(lk + t, links + g);
        } else {
            const int g1 = gy * pitch + gx1;
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                in[q * Lay::IN + t] = __ldg(src + (size_t)q * plane + g);
                in[q * Lay::IN + t + 1] = __ldg(src + (size_t)q * plane + g1);
            }
            lk[t] = __ldg(links + g);
            lk[t + 1] = __ldg(links + g1);
        }
    }
}

template <class S, int TX, int TY, bool FORCE, int NT>
__device__ __forceinline__ void two_steps_persistent(const S *__restrict__ src, S *__restrict__ dst,
                                                     const uint16_t *__restrict__ links, int nx, int ny, int pitch,
                                                     int plane, int periodic, const D2Q9Params &prm,
                                                     unsigned char *smem, int tiles_x, int ntiles) {
    using Lay = Layout<S, TX, TY>;
    using LP = LayoutP<S, TX, TY>;
    static_assert(TX % 2 == 0 && Lay::IW % 2 == 0 && Lay::MW % 2 == 0, "cells go in pairs");
    // input buffer b: its populations at b * buf_bytes, its link words behind them
    auto inb = [&](int b) { return reinterpret_cast<S *>(smem + (size_t)b * LP::buf_bytes); };
    auto lkb = [&](int b) { return reinterpret_cast<uint16_t *>(smem + (size_t)b * LP::buf_bytes + LP::in_bytes); };
    S *mid = reinterpret_cast<S *>(smem + 2 * LP::buf_bytes);
    const bool px = periodic & 1, py = periodic & 2;
    const float om = omega<float>(prm);
    const Vec2<float> F = force<float>(prm), uw = wall_u<float>(prm);

    int t = (int)blockIdx.x, buf = 0;
    if (t < ntiles)
        issue_tile<S, TX, TY, NT>(src, links, nx, ny, pitch, plane, px, py, (t % tiles_x) * TX,
                                  (t / tiles_x) * TY, inb(0), lkb(0));
    copy_async_commit();
    for (; t < ntiles; t += (int)gridDim.x) {
        const int tn = t + (int)gridDim.x;
        if (tn < ntiles)  // the next tile's copies, in flight while this tile is computed
            issue_tile<S, TX, TY, NT>(src, links, nx, ny, pitch, plane, px, py, (tn % tiles_x) * TX,
                                  (tn / tiles_x) * TY, inb(buf ^ 1), lkb(buf ^ 1));
        copy_async_commit();
        copy_async_wait<1>();  // this tile's copies (all but the group just issued)
        __syncthreads();
        const S *in = inb(buf);
        const uint16_t *lk = lkb(buf);
        const int x0 = (t % tiles_x) * TX, y0 = (t / tiles_x) * TY;
        // first step on the tile grown by one cell, two adjacent cells at a time
        for (int k = (int)threadIdx.x; k < Lay::MN / 2; k += NT) {
            const int j = k / (Lay::MW / 2), i = 2 * (k - j * (Lay::MW / 2));
            const int c = (j + 1) * Lay::IW + (i + 1);
            const uint32_t L0 = lk[c], L1 = lk[c + 1];
            float2 h[9];
            gather_pair<S, Lay::IW, Lay::IN>(in, i + 1, j + 1, L0 == LINK_SOLID ? 0u : L0,
                                             L1 == LINK_SOLID ? 0u : L1, uw, h);
            collide_t<S, float2, FORCE>(h, om, F);
            const int m = j * Lay::MW + i;
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                mid[q * Lay::MN + m] = Store<S>::from(h[q].x);
                mid[q * Lay::MN + m + 1] = Store<S>::from(h[q].y);
            }
        }
        __syncthreads();
        // second step on the tile itself, two adjacent cells at a time, into dst
        for (int k = (int)threadIdx.x; k < TX * TY / 2; k += NT) {
            const int j = k / (TX / 2), i = 2 * (k - j * (TX / 2));
            const int x = x0 + i, y = y0 + j;
            if (x >= nx || y >= ny) continue;
            const int c = (j + 2) * Lay::IW + (i + 2);
            const uint32_t L0 = lk[c], L1 = lk[c + 1];
            const bool w0 = L0 != LINK_SOLID, w1 = x + 1 < nx && L1 != LINK_SOLID;
            if (!w0 && !w1) continue;
            float2 h[9];
            gather_pair<S, Lay::MW, Lay::MN>(mid, i + 1, j + 1, w0 ? L0 : 0u, w1 ? L1 : 0u, uw, h);
            collide_t<S, float2, FORCE>(h, om, F);
            const int g = y * pitch + x;
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                if (w0) dst[(size_t)q * plane + g] = Store<S>::from(h[q].x);
                if (w1) dst[(size_t)q * plane + g + 1] = Store<S>::from(h[q].y);
            }
        }
        __syncthreads();  // every thread is done with this buffer and with mid
        buf ^= 1;
    }
    copy_async_wait<0>();  // nothing left in flight when the block ends
}

}  // namespace tile2
}  // namespace d2q9
}  // namespace lbm
