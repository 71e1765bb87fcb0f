// Vectorised D2Q9 update: one thread updates V consecutive cells of a row with V-wide loads and
// stores of every population plane (values in storage space, see d2q9_core.cuh).  The x-1 / x+1
// neighbours that fall outside the thread's vector come from the adjacent lane by warp shuffle;
// lane 0 loads its left neighbour itself (wrapped at x = 0 in a periodic row) and lane 31 its right
// one.  In a periodic row, the vector holding the last column patches that cell's three values from
// x = 0.  Cells with bounce-back links take their own opposite population (one extra wide load per
// population that bounces somewhere in the vector); solid cells copy their own populations, so both
// A/B buffers keep identical values there.  Elements beyond the last column compute garbage that is
// stored only into the row padding, which no cell ever reads.
//
// All 32 lanes of a warp must call step_vec for the same row with consecutive vectors, lane 0
// holding a vector that starts on a multiple of 32 * V (the shuffles use the full mask): blockDim.x
// is a multiple of 32, and threads beyond the row load clamped addresses and store nothing.
#pragma once

#include "d2q9_core.cuh"

namespace lbm {
namespace d2q9 {

template <class S, class I>
__device__ __forceinline__ void scalar_cell(const S *__restrict__ src, S *__restrict__ dst,
                                            const uint16_t *__restrict__ links, int x, int y, int nx, int ny,
                                            I pitch, I plane, int periodic, const D2Q9Params &prm, bool force) {
    using R = typename Store<S>::R;
    const I c = (I)y * pitch + x;
    const uint32_t L = __ldg(links + c);
    if (L == LINK_SOLID) return;
    R h[9];
    gather<S, R>(src, L, x, y, nx, ny, (int64_t)pitch, (int64_t)plane, periodic, wall_u<R>(prm), h);
    if (force)
        collide<S, R, true>(h, omega<R>(prm), d2q9::force<R>(prm));
    else
        collide<S, R, false>(h, omega<R>(prm), d2q9::force<R>(prm));
#pragma unroll
    for (int q = 0; q < 9; ++q) sth<S>(dst + q * plane + c, h[q]);
}

// The source values one thread reads for its vector of a row, kept as raw stored words until
// they are used: a thread can hold the next row's loads in flight while it updates this row
// (16-bit storage: 9 populations x V cells in 9 V / 2 registers).
template <class S, int V, class I>
struct RowLoad {
    using T = typename RawPack<sizeof(S) * V>::T;
    using LT = typename RawPack<2 * V < 4 ? 4 : 2 * V>::T;
    T q0, q2, q4, a1, a5, a8, b3, b6, b7;  // populations at x0 .. x0+V-1 of rows y (0, 1, 3), y-1 (2, 5, 6), y+1 (4, 7, 8)
    LT links;
    S e[3];   // lane 0: populations 1, 5, 8 at x0 - 1; lane 31: populations 3, 6, 7 at x0 + V
              // (flat mapping: the left edge only)
    S er[3];  // flat mapping: populations 3, 6, 7 at x0 + V
    S w[3];   // periodic row, the vector holding the last column: populations 3, 6, 7 at x = 0
    I r0, rm, rp;
    int xa;
};

template <class T, int POL>
__device__ __forceinline__ T ld_raw(const T *p, uint64_t pol) {
    if constexpr (POL == 0)
        return __ldg(p);
    else
        return ld_hint<T>(p, pol);
}

template <class S, int V, class I, int POL>
__device__ __forceinline__ void load_row(RowLoad<S, V, I> &ld, const S *__restrict__ src,
                                         const uint16_t *__restrict__ links, int x0, int y, int nx, int ny, I pitch,
                                         I plane, int periodic, uint64_t pol_ld) {
    using T = typename RowLoad<S, V, I>::T;
    using LT = typename RowLoad<S, V, I>::LT;
    const int lane = threadIdx.x & 31;
    const int xa = min(x0, (int)pitch - V);  // threads beyond the row load a valid vector
    int ym = y - 1, yp = y + 1;
    if (ym < 0) ym = (periodic & 2) ? ny - 1 : 0;
    if (yp >= ny) yp = (periodic & 2) ? 0 : ny - 1;
    const I r0 = (I)y * pitch, rm = (I)ym * pitch, rp = (I)yp * pitch;
    ld.r0 = r0;
    ld.rm = rm;
    ld.rp = rp;
    ld.xa = xa;
    auto at = [&](int q, I r) { return reinterpret_cast<const T *>(src + q * plane + r + xa); };
    ld.q0 = ld_raw<T, POL>(at(0, r0), pol_ld);
    ld.q2 = ld_raw<T, POL>(at(2, rm), pol_ld);
    ld.q4 = ld_raw<T, POL>(at(4, rp), pol_ld);
    ld.a1 = ld_raw<T, POL>(at(1, r0), pol_ld);
    ld.a5 = ld_raw<T, POL>(at(5, rm), pol_ld);
    ld.a8 = ld_raw<T, POL>(at(8, rp), pol_ld);
    ld.b3 = ld_raw<T, POL>(at(3, r0), pol_ld);
    ld.b6 = ld_raw<T, POL>(at(6, rm), pol_ld);
    ld.b7 = ld_raw<T, POL>(at(7, rp), pol_ld);
    if constexpr (V == 1)
        ld.links = __ldg(links + r0 + xa);
    else
        ld.links = __ldg(reinterpret_cast<const LT *>(links + r0 + xa));
    if (lane == 0) {
        // from the clamped xa: a warp lying wholly beyond the row must not address past it
        int xm = xa - 1;
        if (xm < 0) xm = (periodic & 1) ? nx - 1 : 0;  // unused (bounce-back) when not periodic
        ld.e[0] = __ldg(src + 1 * plane + r0 + xm);
        ld.e[1] = __ldg(src + 5 * plane + rm + xm);
        ld.e[2] = __ldg(src + 8 * plane + rp + xm);
    } else if (lane == 31) {
        const int xq = min(x0 + V, (int)pitch - 1);
        ld.e[0] = __ldg(src + 3 * plane + r0 + xq);
        ld.e[1] = __ldg(src + 6 * plane + rm + xq);
        ld.e[2] = __ldg(src + 7 * plane + rp + xq);
    }
    const int kl = nx - 1 - x0;
    if ((periodic & 1) && kl >= 0 && kl < V) {
        ld.w[0] = __ldg(src + 3 * plane + r0);
        ld.w[1] = __ldg(src + 6 * plane + rm);
        ld.w[2] = __ldg(src + 7 * plane + rp);
    }
}

// Update the vector of ld and store it to dst.  own(q, out) yields the vector's own population q
// (bounce-back takes the opposite population of the cell itself; solid cells keep their own).
template <class S, int V, bool FORCE, class I, int POL, class Own>
__device__ __forceinline__ void finish_row(const RowLoad<S, V, I> &ld, Own own, S *__restrict__ dst, int x0, int nx,
                                           I plane, int periodic, const D2Q9Params &prm, uint64_t pol_st,
                                           const S (&el)[3], const S (&er)[3], bool left_own, bool right_own,
                                           bool active) {
    using R = typename Store<S>::R;
    const I r0 = ld.r0;
    R f[9][V];
    R a1[V], a5[V], a8[V], b3[V], b6[V], b7[V];
    unpack<S, V>(ld.q0, f[0]);
    unpack<S, V>(ld.q2, f[2]);
    unpack<S, V>(ld.q4, f[4]);
    unpack<S, V>(ld.a1, a1);
    unpack<S, V>(ld.a5, a5);
    unpack<S, V>(ld.a8, a8);
    unpack<S, V>(ld.b3, b3);
    unpack<S, V>(ld.b6, b6);
    unpack<S, V>(ld.b7, b7);
    uint32_t L[V];
    if constexpr (V == 1) {
        L[0] = ld.links;
    } else {
        uint16_t e[V];
        memcpy(e, &ld.links, sizeof(e));
#pragma unroll
        for (int k = 0; k < V; ++k) L[k] = e[k];
    }

    // populations moving +x come from x-1: the previous lane's last element
    R p1 = __shfl_up_sync(0xffffffffu, a1[V - 1], 1);
    R p5 = __shfl_up_sync(0xffffffffu, a5[V - 1], 1);
    R p8 = __shfl_up_sync(0xffffffffu, a8[V - 1], 1);
    // populations moving -x come from x+V: the next lane's first element
    R n3 = __shfl_down_sync(0xffffffffu, b3[0], 1);
    R n6 = __shfl_down_sync(0xffffffffu, b6[0], 1);
    R n7 = __shfl_down_sync(0xffffffffu, b7[0], 1);
    if (left_own) {
        p1 = Store<S>::to(el[0]);
        p5 = Store<S>::to(el[1]);
        p8 = Store<S>::to(el[2]);
    }
    if (right_own) {
        n3 = Store<S>::to(er[0]);
        n6 = Store<S>::to(er[1]);
        n7 = Store<S>::to(er[2]);
    }
#pragma unroll
    for (int k = 0; k < V; ++k) {
        f[1][k] = k == 0 ? p1 : a1[k - 1];
        f[5][k] = k == 0 ? p5 : a5[k - 1];
        f[8][k] = k == 0 ? p8 : a8[k - 1];
        f[3][k] = k == V - 1 ? n3 : b3[k + 1];
        f[6][k] = k == V - 1 ? n6 : b6[k + 1];
        f[7][k] = k == V - 1 ? n7 : b7[k + 1];
    }
    // periodic row: the last column pulls q = 3, 6, 7 from x = 0
    const int kl = nx - 1 - x0;
    if ((periodic & 1) && kl >= 0 && kl < V) {
        const R w3 = Store<S>::to(ld.w[0]), w6 = Store<S>::to(ld.w[1]), w7 = Store<S>::to(ld.w[2]);
#pragma unroll
        for (int k = 0; k < V; ++k)
            if (k == kl) {
                f[3][k] = w3;
                f[6][k] = w6;
                f[7][k] = w7;
            }
    }

    uint32_t any = 0;
#pragma unroll
    for (int k = 0; k < V; ++k) any |= L[k];
    bool solid_any = false;
    if (any) {
        const Vec2<R> uw = wall_u<R>(prm);
#pragma unroll
        for (int q = 1; q < 9; ++q) {
            uint32_t hit = 0;
#pragma unroll
            for (int k = 0; k < V; ++k) hit |= L[k] != LINK_SOLID ? (L[k] >> (q - 1)) & 1u : 0u;
            if (hit) {
                R mine[V];
                own(opp(q), mine);
#pragma unroll
                for (int k = 0; k < V; ++k) {
                    if (L[k] != LINK_SOLID && ((L[k] >> (q - 1)) & 1u)) {
                        R v = mine[k];
                        if ((L[k] >> (q + 7)) & 1u) v = add_(v, wall_term<S, R>(q, uw));
                        f[q][k] = v;
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < V; ++k) solid_any |= L[k] == LINK_SOLID;
    }

    if constexpr (std::is_same<R, float>::value && V % 2 == 0) {
        // FP32 arithmetic: cells k and k + 1 collide together on the packed FP32 pipe
#pragma unroll
        for (int k = 0; k < V; k += 2) {
            float2 h[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) h[q] = make_float2(f[q][k], f[q][k + 1]);
            collide_t<S, float2, FORCE>(h, omega<R>(prm), force<R>(prm));
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                f[q][k] = h[q].x;
                f[q][k + 1] = h[q].y;
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < V; ++k) {
            R h[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) h[q] = f[q][k];
            collide<S, R, FORCE>(h, omega<R>(prm), force<R>(prm));
#pragma unroll
            for (int q = 0; q < 9; ++q) f[q][k] = h[q];
        }
    }

    if (!active || x0 >= nx) return;  // vector entirely in the row padding (or past the end of a flat tile)
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        if (solid_any) {
            R mine[V];
            own(q, mine);
#pragma unroll
            for (int k = 0; k < V; ++k)
                if (L[k] == LINK_SOLID) f[q][k] = mine[k];
        }
        st_pack_pol<S, V, POL>(dst + q * plane + r0 + x0, f[q], pol_st);
    }
}

template <class S, int V, bool FORCE, class I, int POL = 0>
__device__ __forceinline__ void step_vec(const S *__restrict__ src, S *__restrict__ dst,
                                         const uint16_t *__restrict__ links, int x0, int y, int nx, int ny,
                                         I pitch, I plane, int periodic, const D2Q9Params &prm) {
    const uint64_t pol_ld = POL ? policy_evict_first() : 0;
    const uint64_t pol_st = POL == 1 ? policy_evict_last() : 0;
    RowLoad<S, V, I> ld;
    load_row<S, V, I, POL>(ld, src, links, x0, y, nx, ny, pitch, plane, periodic, pol_ld);
    // own populations at the clamped xa (equal to x0 for every vector that is stored)
    const S *mine = src + ld.r0 + ld.xa;
    auto own = [&](int q, typename Store<S>::R (&out)[V]) { ld_pack<S, V>(mine + q * plane, out); };
    const int lane = threadIdx.x & 31;
    finish_row<S, V, FORCE, I, POL>(ld, own, dst, x0, nx, plane, periodic, prm, pol_st, ld.e, ld.e, lane == 0,
                                    lane == 31, true);
}

// Flat mapping (the batch kernel): the 32 lanes of a warp hold 32 consecutive vectors of the slot's
// padded cell array [0, pitch * ny), row after row, so a warp may span rows.  The caller gives each
// lane its own (x0, y) with x0 a multiple of V below pitch (a vector never straddles rows, pitch
// being a multiple of 32).  A lane takes its x - 1 neighbours from the previous lane unless it starts
// a row or is lane 0 (left_own: it loads them, wrapped or clamped at x = 0 as above), and its x + V
// neighbours from the next lane unless it ends a padded row or is lane 31 (right_own).  Lanes past
// the slot's last vector are given that vector and active = false: they load in bounds, take part
// in the shuffles and store nothing.  Per cell the arithmetic is that of step_vec, so the results
// are bit-identical to the row mapping and to the single-domain kernel.
template <class S, int V, class I>
__device__ __forceinline__ void load_row_flat(RowLoad<S, V, I> &ld, const S *__restrict__ src,
                                              const uint16_t *__restrict__ links, int x0, int y, int nx, int ny,
                                              I pitch, I plane, int periodic, bool left_own, bool right_own) {
    using T = typename RowLoad<S, V, I>::T;
    using LT = typename RowLoad<S, V, I>::LT;
    int ym = y - 1, yp = y + 1;
    if (ym < 0) ym = (periodic & 2) ? ny - 1 : 0;
    if (yp >= ny) yp = (periodic & 2) ? 0 : ny - 1;
    const I r0 = (I)y * pitch, rm = (I)ym * pitch, rp = (I)yp * pitch;
    ld.r0 = r0;
    ld.rm = rm;
    ld.rp = rp;
    ld.xa = x0;
    auto at = [&](int q, I r) { return reinterpret_cast<const T *>(src + q * plane + r + x0); };
    ld.q0 = __ldg(at(0, r0));
    ld.q2 = __ldg(at(2, rm));
    ld.q4 = __ldg(at(4, rp));
    ld.a1 = __ldg(at(1, r0));
    ld.a5 = __ldg(at(5, rm));
    ld.a8 = __ldg(at(8, rp));
    ld.b3 = __ldg(at(3, r0));
    ld.b6 = __ldg(at(6, rm));
    ld.b7 = __ldg(at(7, rp));
    if constexpr (V == 1)
        ld.links = __ldg(links + r0 + x0);
    else
        ld.links = __ldg(reinterpret_cast<const LT *>(links + r0 + x0));
    if (left_own) {
        int xm = x0 - 1;
        if (xm < 0) xm = (periodic & 1) ? nx - 1 : 0;  // unused (bounce-back) when not periodic
        ld.e[0] = __ldg(src + 1 * plane + r0 + xm);
        ld.e[1] = __ldg(src + 5 * plane + rm + xm);
        ld.e[2] = __ldg(src + 8 * plane + rp + xm);
    }
    if (right_own) {
        const int xq = min(x0 + V, (int)pitch - 1);
        ld.er[0] = __ldg(src + 3 * plane + r0 + xq);
        ld.er[1] = __ldg(src + 6 * plane + rm + xq);
        ld.er[2] = __ldg(src + 7 * plane + rp + xq);
    }
    const int kl = nx - 1 - x0;
    if ((periodic & 1) && kl >= 0 && kl < V) {
        ld.w[0] = __ldg(src + 3 * plane + r0);
        ld.w[1] = __ldg(src + 6 * plane + rm);
        ld.w[2] = __ldg(src + 7 * plane + rp);
    }
}

template <class S, int V, bool FORCE, class I>
__device__ __forceinline__ void step_vec_flat(const S *__restrict__ src, S *__restrict__ dst,
                                              const uint16_t *__restrict__ links, int x0, int y, int nx, int ny,
                                              I pitch, I plane, int periodic, const D2Q9Params &prm, bool active) {
    const int lane = threadIdx.x & 31;
    const bool left_own = lane == 0 || x0 == 0;
    const bool right_own = lane == 31 || x0 + V == (int)pitch;
    RowLoad<S, V, I> ld;
    load_row_flat<S, V, I>(ld, src, links, x0, y, nx, ny, pitch, plane, periodic, left_own, right_own);
    const S *mine = src + ld.r0 + x0;
    auto own = [&](int q, typename Store<S>::R (&out)[V]) { ld_pack<S, V>(mine + q * plane, out); };
    finish_row<S, V, FORCE, I, 0>(ld, own, dst, x0, nx, plane, periodic, prm, 0, ld.e, ld.er, left_own, right_own,
                                  active);
}

}  // namespace d2q9
}  // namespace lbm
