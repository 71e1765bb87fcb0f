// Two D2Q9 time steps per launch on a shared-memory tile (temporal blocking).
//
// A block owns an output tile of TX x TY cells.  It loads the source populations of the tile and a
// halo of two cells on every side (the tile grown by 2: what two pull steps reach), computes the
// first step for the tile grown by 1 into a second shared-memory tile, and the second step for the
// tile itself into the destination buffer.  The populations are read from and written to HBM once
// per two updates; the halo's first-step cells are computed by both neighbouring blocks.
//
// Per cell the update is scalar_cell()'s (d2q9_vec.cuh) -- the same pulls, bounce-back and
// moving-wall terms, and the same collide() -- and the first step's values are held in the storage
// type, rounded as the one-step kernel stores them, so two steps here are bit-identical to two
// launches of the one-step kernels.  Solid cells are not written (their values are never read:
// a pull from a solid cell is replaced by bounce-back).  Halo cells outside a non-periodic domain
// are loaded from a clamped position and never computed: a cell at the domain edge replaces every
// pull from outside by bounce-back.
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

// populations of the cell at (ci, cj) of a tile T[9][H][W] (row width W), its pulls from
// (ci - c_x, cj - c_y), replaced by its own opposite population where link bit q - 1 is set (plus
// the moving-wall term where bit q + 7 is)
template <class S, class R, int W, int N>
__device__ __forceinline__ void gather_tile(const S *T, int ci, int cj, uint32_t L, Vec2<R> uw, R h[9]) {
    const int c = cj * W + ci;
#pragma unroll
    for (int q = 0; q < 9; ++q) h[q] = Store<S>::to(T[q * N + c - cy(q) * W - cx(q)]);
    if (L) {
#pragma unroll
        for (int q = 1; q < 9; ++q) {
            if (L & (1u << (q - 1))) {
                R v = Store<S>::to(T[opp(q) * N + c]);
                if (L & (1u << (q + 7))) v = add_(v, wall_term<S, R>(q, uw));
                h[q] = v;
            }
        }
    }
}

template <class S, int TX, int TY, bool FORCE>
__device__ __forceinline__ void two_steps(const S *__restrict__ src, S *__restrict__ dst,
                                          const uint16_t *__restrict__ links, int nx, int ny, int pitch,
                                          int plane, int periodic, const D2Q9Params &prm, unsigned char *smem) {
    using R = typename Store<S>::R;
    using Lay = Layout<S, TX, TY>;
    S *in = reinterpret_cast<S *>(smem);
    S *mid = reinterpret_cast<S *>(smem + Lay::in_bytes);
    uint16_t *lk = reinterpret_cast<uint16_t *>(smem + Lay::in_bytes + Lay::mid_bytes);
    const int x0 = (int)blockIdx.x * TX, y0 = (int)blockIdx.y * TY;
    const bool px = periodic & 1, py = periodic & 2;

    // the source tile with its two-cell halo (wrapped when periodic, clamped otherwise)
    for (int k = (int)threadIdx.x; k < Lay::IN; k += THREADS) {
        const int j = k / Lay::IW, i = k - j * Lay::IW;
        bool inside = true;
        const int gx = wrap_or_clamp(x0 - 2 + i, nx, px, inside);
        const int gy = wrap_or_clamp(y0 - 2 + j, ny, py, inside);
        const int g = gy * pitch + gx;
#pragma unroll
        for (int q = 0; q < 9; ++q) in[q * Lay::IN + k] = __ldg(src + (size_t)q * plane + g);
    }
    // the link words of the first step's tile; 0xFFFF marks a cell outside the domain
    for (int k = (int)threadIdx.x; k < Lay::MN; k += THREADS) {
        const int j = k / Lay::MW, i = k - j * Lay::MW;
        bool inside = true;
        const int gx = wrap_or_clamp(x0 - 1 + i, nx, px, inside);
        const int gy = wrap_or_clamp(y0 - 1 + j, ny, py, inside);
        lk[k] = inside ? __ldg(links + gy * pitch + gx) : (uint16_t)0xFFFF;
    }
    __syncthreads();

    const R om = omega<R>(prm);
    const Vec2<R> F = force<R>(prm), uw = wall_u<R>(prm);
    // first step: the tile grown by one cell (mid cell (i, j) is in-tile cell (i + 1, j + 1))
    for (int k = (int)threadIdx.x; k < Lay::MN; k += THREADS) {
        const uint32_t L = lk[k];
        if (L == 0xFFFFu || L == LINK_SOLID) continue;  // outside the domain, or solid: never read
        const int j = k / Lay::MW, i = k - j * Lay::MW;
        R h[9];
        gather_tile<S, R, Lay::IW, Lay::IN>(in, i + 1, j + 1, L, uw, h);
        collide<S, R, FORCE>(h, om, F);
#pragma unroll
        for (int q = 0; q < 9; ++q) mid[q * Lay::MN + k] = Store<S>::from(h[q]);
    }
    __syncthreads();

    // second step: the tile itself (output cell (i, j) is mid cell (i + 1, j + 1)), into dst
    for (int k = (int)threadIdx.x; k < TX * TY; k += THREADS) {
        const int j = k / TX, i = k - j * TX;
        const int x = x0 + i, y = y0 + j;
        if (x >= nx || y >= ny) continue;
        const int m = (j + 1) * Lay::MW + (i + 1);
        const uint32_t L = lk[m];
        if (L == LINK_SOLID) continue;
        R h[9];
        gather_tile<S, R, Lay::MW, Lay::MN>(mid, i + 1, j + 1, L, uw, h);
        collide<S, R, FORCE>(h, om, F);
        const int g = y * pitch + x;
#pragma unroll
        for (int q = 0; q < 9; ++q) dst[(size_t)q * plane + g] = Store<S>::from(h[q]);
    }
}

}  // namespace tile2
}  // namespace d2q9
}  // namespace lbm
