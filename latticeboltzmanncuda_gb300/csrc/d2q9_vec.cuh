// Vectorised D2Q9 update: one thread updates V consecutive cells of a row with V-wide loads and
// stores of every population plane (values in storage space, see d2q9_core.cuh).  The x-1 / x+1
// neighbours that fall outside the thread's vector come from the adjacent lane by warp shuffle;
// lane 0 loads its left neighbour itself (wrapped at x = 0 in a periodic row) and lane 31 its right
// one.  In a periodic row, the vector holding the last column patches that cell's three values from
// x = 0.  Cells with bounce-back links take their own opposite population (one extra wide load per
// population that bounces somewhere in the vector, none for populations 1 and 3, whose own values
// are loaded for the pull); solid cells are not written (both buffers agree there).  Elements beyond
// the last column compute garbage that is stored only into the row padding, which no cell ever reads.
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

// POL 0: read-only path; 1, 2: read-only path with an L2 eviction hint; 3: loads at L2 (`.cg`),
// coherent with the stores of other blocks earlier in the same kernel (the persistent batch
// kernel, whose steps follow one another inside one launch)
template <class T, int POL>
__device__ __forceinline__ T ld_raw(const T *p, uint64_t pol) {
    if constexpr (POL == 0)
        return __ldg(p);
    else if constexpr (POL == 3)
        return __ldcg(p);
    else
        return ld_hint<T>(p, pol);
}
template <int POL, class T>
__device__ __forceinline__ T ld_one(const T *p) {
    if constexpr (POL == 3)
        return __ldcg(p);
    else
        return __ldg(p);
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
        ld.e[0] = ld_one<POL>(src + 1 * plane + r0 + xm);
        ld.e[1] = ld_one<POL>(src + 5 * plane + rm + xm);
        ld.e[2] = ld_one<POL>(src + 8 * plane + rp + xm);
    } else if (lane == 31) {
        const int xq = min(x0 + V, (int)pitch - 1);
        ld.e[0] = ld_one<POL>(src + 3 * plane + r0 + xq);
        ld.e[1] = ld_one<POL>(src + 6 * plane + rm + xq);
        ld.e[2] = ld_one<POL>(src + 7 * plane + rp + xq);
    }
    const int kl = nx - 1 - x0;
    if ((periodic & 1) && kl >= 0 && kl < V) {
        ld.w[0] = ld_one<POL>(src + 3 * plane + r0);
        ld.w[1] = ld_one<POL>(src + 6 * plane + rm);
        ld.w[2] = ld_one<POL>(src + 7 * plane + rp);
    }
}

// Words of a raw pack: 16-bit storage holds two cells per 32-bit word (cell 2j in the low half).
template <int NW, class T>
__device__ __forceinline__ void words(const T &raw, uint32_t (&w)[NW]) {
    static_assert(sizeof(T) == 4 * NW, "pack size");
    memcpy(w, &raw, sizeof(w));
}
template <class S>
__device__ __forceinline__ uint32_t raw16(S v) {
    uint16_t u;
    memcpy(&u, &v, sizeof(u));
    return u;
}
// (high half of a, low half of b): a pair shifted by one cell across two adjacent words
__device__ __forceinline__ uint32_t hi_lo(uint32_t a, uint32_t b) { return __byte_perm(a, b, 0x5432); }
// 0xFFFF in each 16-bit half of a link word whose bit q - 1 is set: the bit is moved to the sign
// position of byte 0 (byte 2 for the high half) and prmt replicates each sign over its half
__device__ __forceinline__ uint32_t link_halves(uint32_t lw, int q) {
    uint32_t m;
    asm("prmt.b32 %0, %1, 0, 0xAA88;" : "=r"(m) : "r"(lw << (8 - q)));
    return m;
}
// 16-bit storage: bit k of the result is set when cell k of the vector is solid
template <int NW>
__device__ __forceinline__ uint32_t solid_cells(const uint32_t (&lw)[NW]) {
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < NW; ++j)
        s |= ((lw[j] & 0xFFFFu) == LINK_SOLID ? 1u : 0u) << (2 * j) | ((lw[j] >> 16) == LINK_SOLID ? 1u : 0u) << (2 * j + 1);
    return s;
}

// Update the vector of ld and store it to dst.  own(q) returns the raw pack of the vector's own
// population q (bounce-back takes the opposite population of the cell itself).  Solid cells are
// not written: no fluid cell reads their values (a pull from a solid cell is replaced by
// bounce-back), and both buffers hold the same values there (the initialisation and the population
// upload write both, the link build copies every solid cell into the other buffer, a checkpoint is
// restored into both), so a vector without solid cells is stored whole, a mixed vector cell by
// cell, an all-solid one not at all.
//
// 16-bit storage assembles the pulled populations and applies the bounce-back on the raw pairs:
// the x-shifted vectors are byte permutes of adjacent words, and a bounce-back is one select per
// pair under a mask built from the link word.  The arithmetic values are then those of the float
// path (a raw select followed by the conversion is the conversion followed by the select); each
// pair of cells is unpacked, collided and packed back in turn, so at most 18 FP32 values are live.
template <class S, int V, bool FORCE, class I, int POL, class Own>
__device__ __forceinline__ void finish_row(const RowLoad<S, V, I> &ld, Own own, S *__restrict__ dst, int x0, int nx,
                                           I plane, int periodic, const D2Q9Params &prm, uint64_t pol_st,
                                           const S (&el)[3], const S (&er)[3], bool left_own, bool right_own,
                                           bool active) {
    using R = typename Store<S>::R;
    using T = typename RowLoad<S, V, I>::T;
    const I r0 = ld.r0;
    constexpr bool RAW = sizeof(S) == 2 && V % 2 == 0;  // 16-bit storage: the raw-pair path
    R f[9][V];
    uint32_t solid = 0;
    const int kl = nx - 1 - x0;  // the vector's element holding the last column, if in [0, V)
    if constexpr (RAW) {
        constexpr int NW = V / 2;
        uint32_t P[9][NW], A1[NW], A5[NW], A8[NW], B3[NW], B6[NW], B7[NW], LW[NW];
        words<NW>(ld.q0, P[0]);
        words<NW>(ld.q2, P[2]);
        words<NW>(ld.q4, P[4]);
        words<NW>(ld.a1, A1);
        words<NW>(ld.a5, A5);
        words<NW>(ld.a8, A8);
        words<NW>(ld.b3, B3);
        words<NW>(ld.b6, B6);
        words<NW>(ld.b7, B7);
        words<NW>(ld.links, LW);
        // +x populations from x - 1: the previous lane's last cell (high half of its last word);
        // -x populations from x + V: the next lane's first cell (low half of its first word)
        uint32_t p1 = __shfl_up_sync(0xffffffffu, A1[NW - 1], 1);
        uint32_t p5 = __shfl_up_sync(0xffffffffu, A5[NW - 1], 1);
        uint32_t p8 = __shfl_up_sync(0xffffffffu, A8[NW - 1], 1);
        uint32_t n3 = __shfl_down_sync(0xffffffffu, B3[0], 1);
        uint32_t n6 = __shfl_down_sync(0xffffffffu, B6[0], 1);
        uint32_t n7 = __shfl_down_sync(0xffffffffu, B7[0], 1);
        if (left_own) {
            p1 = raw16(el[0]) << 16;
            p5 = raw16(el[1]) << 16;
            p8 = raw16(el[2]) << 16;
        }
        if (right_own) {
            n3 = raw16(er[0]);
            n6 = raw16(er[1]);
            n7 = raw16(er[2]);
        }
#pragma unroll
        for (int j = 0; j < NW; ++j) {
            P[1][j] = hi_lo(j == 0 ? p1 : A1[j - 1], A1[j]);
            P[5][j] = hi_lo(j == 0 ? p5 : A5[j - 1], A5[j]);
            P[8][j] = hi_lo(j == 0 ? p8 : A8[j - 1], A8[j]);
            P[3][j] = hi_lo(B3[j], j + 1 < NW ? B3[j + 1] : n3);
            P[6][j] = hi_lo(B6[j], j + 1 < NW ? B6[j + 1] : n6);
            P[7][j] = hi_lo(B7[j], j + 1 < NW ? B7[j + 1] : n7);
        }
        // periodic row: the last column pulls q = 3, 6, 7 from x = 0
        if ((periodic & 1) && kl >= 0 && kl < V) {
            const uint32_t w3 = raw16(ld.w[0]), w6 = raw16(ld.w[1]), w7 = raw16(ld.w[2]);
            const bool hi = kl & 1;
            const uint32_t keep = hi ? 0x0000FFFFu : 0xFFFF0000u;
#pragma unroll
            for (int j = 0; j < NW; ++j)
                if ((kl >> 1) == j) {
                    P[3][j] = (P[3][j] & keep) | (hi ? w3 << 16 : w3);
                    P[6][j] = (P[6][j] & keep) | (hi ? w6 << 16 : w6);
                    P[7][j] = (P[7][j] & keep) | (hi ? w7 << 16 : w7);
                }
        }
        // bounce-back (link bits 0-7 and 16-23 of a word; solid cells have none)
        uint32_t links = 0;
#pragma unroll
        for (int j = 0; j < NW; ++j) links |= LW[j];
        if (links & 0x00FF00FFu) {
#pragma unroll
            for (int q = 1; q < 9; ++q) {
                if (links & (0x00010001u << (q - 1))) {
                    uint32_t O[NW];
                    // own populations 1 and 3 are the values loaded for the pull (row y)
                    if (opp(q) == 1) {
#pragma unroll
                        for (int j = 0; j < NW; ++j) O[j] = A1[j];
                    } else if (opp(q) == 3) {
#pragma unroll
                        for (int j = 0; j < NW; ++j) O[j] = B3[j];
                    } else {
                        words<NW>(own(opp(q)), O);
                    }
#pragma unroll
                    for (int j = 0; j < NW; ++j) {
                        const uint32_t m = link_halves(LW[j], q);
                        P[q][j] = (P[q][j] & ~m) | (O[j] & m);
                    }
                }
            }
        }
        // moving walls: the wall term on the bounced populations (bit q + 7 with bit q - 1)
        uint32_t wall = 0;
#pragma unroll
        for (int j = 0; j < NW; ++j) wall |= LW[j] & (LW[j] << 8);
        wall &= 0xFF00FF00u;
        // collide pair by pair (cells 2j, 2j + 1 on the packed FP32 pipe), the results packed back
        // into P: at most one pair of cells is held in FP32 at a time
#pragma unroll
        for (int j = 0; j < NW; ++j) {
            float2 h[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                typename Pair<S>::P h2;
                memcpy(&h2, &P[q][j], sizeof(h2));
                h[q] = Pair<S>::to(h2);
            }
            if (wall) {
                const Vec2<R> uw = wall_u<R>(prm);
#pragma unroll
                for (int q = 1; q < 9; ++q) {
                    if (wall & (0x01000100u << (q - 1))) {
                        const R wt = wall_term<S, R>(q, uw);
                        const uint32_t lw = LW[j];
                        if ((lw >> (q - 1)) & (lw >> (q + 7)) & 1u) h[q].x = add_(h[q].x, wt);
                        if ((lw >> (q + 15)) & (lw >> (q + 23)) & 1u) h[q].y = add_(h[q].y, wt);
                    }
                }
            }
            uint32_t rounded[5];  // populations 0-4 come back packed from the conservative rounding
            collide_t<S, float2, FORCE>(h, omega<R>(prm), force<R>(prm), rounded);
#pragma unroll
            for (int q = 0; q < 5; ++q) P[q][j] = rounded[q];
#pragma unroll
            for (int q = 5; q < 9; ++q) {
                const typename Pair<S>::P h2 = Pair<S>::from(h[q].x, h[q].y);
                memcpy(&P[q][j], &h2, sizeof(h2));
            }
        }
        if (!active || x0 >= nx) return;  // vector in the row padding (or past the end of a flat tile)
        solid = solid_cells<NW>(LW);
        if (solid == 0) {
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                T raw;
                memcpy(&raw, P[q], sizeof(raw));
                st_raw_pol<T, POL>(reinterpret_cast<T *>(dst + q * plane + r0 + x0), raw, pol_st);
            }
        } else if (solid != (1u << V) - 1) {
            // mixed vector: the fluid cells one by one
            uint16_t *d16 = reinterpret_cast<uint16_t *>(dst + r0 + x0);
#pragma unroll
            for (int q = 0; q < 9; ++q)
#pragma unroll
                for (int k = 0; k < V; ++k)
                    if (!((solid >> k) & 1u)) d16[q * plane + k] = (uint16_t)(P[q][k >> 1] >> (16 * (k & 1)));
        }
        return;
    } else {
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

        uint32_t any = 0;  // bounce-back bits 0-7 (solid cells have none)
#pragma unroll
        for (int k = 0; k < V; ++k) {
            solid |= (L[k] == LINK_SOLID ? 1u : 0u) << k;
            any |= L[k];
        }
        if (any & 0xFFu) {
            const Vec2<R> uw = wall_u<R>(prm);
#pragma unroll
            for (int q = 1; q < 9; ++q) {
                if ((any >> (q - 1)) & 1u) {
                    R mine[V];
                    if (opp(q) == 1) {
#pragma unroll
                        for (int k = 0; k < V; ++k) mine[k] = a1[k];
                    } else if (opp(q) == 3) {
#pragma unroll
                        for (int k = 0; k < V; ++k) mine[k] = b3[k];
                    } else {
                        unpack<S, V>(own(opp(q)), mine);
                    }
#pragma unroll
                    for (int k = 0; k < V; ++k) {
                        if ((L[k] >> (q - 1)) & 1u) {
                            R v = mine[k];
                            if ((L[k] >> (q + 7)) & 1u) v = add_(v, wall_term<S, R>(q, uw));
                            f[q][k] = v;
                        }
                    }
                }
            }
        }
    }
    if constexpr (RAW) return;  // collided and stored above

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
    if (solid == 0) {
#pragma unroll
        for (int q = 0; q < 9; ++q) st_pack_pol<S, V, POL>(dst + q * plane + r0 + x0, f[q], pol_st);
    } else if (solid != (1u << V) - 1) {
        // mixed vector: the fluid cells one by one
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            T raw;
            pack<S, V>(f[q], raw);
            S e[V];
            memcpy(e, &raw, sizeof(e));
#pragma unroll
            for (int k = 0; k < V; ++k)
                if (!((solid >> k) & 1u)) dst[q * plane + r0 + x0 + k] = e[k];
        }
    }
}

template <class S, int V, bool FORCE, class I, int POL = 0>
__device__ __forceinline__ void step_vec(const S *__restrict__ src, S *__restrict__ dst,
                                         const uint16_t *__restrict__ links, int x0, int y, int nx, int ny,
                                         I pitch, I plane, int periodic, const D2Q9Params &prm) {
    const uint64_t pol_ld = POL == 1 || POL == 2 ? policy_evict_first() : 0;
    const uint64_t pol_st = POL == 1 ? policy_evict_last() : 0;
    RowLoad<S, V, I> ld;
    load_row<S, V, I, POL>(ld, src, links, x0, y, nx, ny, pitch, plane, periodic, pol_ld);
    // own populations at the clamped xa (equal to x0 for every vector that is stored)
    const S *mine = src + ld.r0 + ld.xa;
    using T = typename RowLoad<S, V, I>::T;
    auto own = [&](int q) { return ld_one<POL>(reinterpret_cast<const T *>(mine + q * plane)); };
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
template <class S, int V, class I, int POL = 0>
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
    ld.q0 = ld_one<POL>(at(0, r0));
    ld.q2 = ld_one<POL>(at(2, rm));
    ld.q4 = ld_one<POL>(at(4, rp));
    ld.a1 = ld_one<POL>(at(1, r0));
    ld.a5 = ld_one<POL>(at(5, rm));
    ld.a8 = ld_one<POL>(at(8, rp));
    ld.b3 = ld_one<POL>(at(3, r0));
    ld.b6 = ld_one<POL>(at(6, rm));
    ld.b7 = ld_one<POL>(at(7, rp));
    if constexpr (V == 1)
        ld.links = __ldg(links + r0 + x0);
    else
        ld.links = __ldg(reinterpret_cast<const LT *>(links + r0 + x0));
    if (left_own) {
        int xm = x0 - 1;
        if (xm < 0) xm = (periodic & 1) ? nx - 1 : 0;  // unused (bounce-back) when not periodic
        ld.e[0] = ld_one<POL>(src + 1 * plane + r0 + xm);
        ld.e[1] = ld_one<POL>(src + 5 * plane + rm + xm);
        ld.e[2] = ld_one<POL>(src + 8 * plane + rp + xm);
    }
    if (right_own) {
        const int xq = min(x0 + V, (int)pitch - 1);
        ld.er[0] = ld_one<POL>(src + 3 * plane + r0 + xq);
        ld.er[1] = ld_one<POL>(src + 6 * plane + rm + xq);
        ld.er[2] = ld_one<POL>(src + 7 * plane + rp + xq);
    }
    const int kl = nx - 1 - x0;
    if ((periodic & 1) && kl >= 0 && kl < V) {
        ld.w[0] = ld_one<POL>(src + 3 * plane + r0);
        ld.w[1] = ld_one<POL>(src + 6 * plane + rm);
        ld.w[2] = ld_one<POL>(src + 7 * plane + rp);
    }
}

template <class S, int V, bool FORCE, class I, int POL = 0>
__device__ __forceinline__ void step_vec_flat(const S *__restrict__ src, S *__restrict__ dst,
                                              const uint16_t *__restrict__ links, int x0, int y, int nx, int ny,
                                              I pitch, I plane, int periodic, const D2Q9Params &prm, bool active) {
    const int lane = threadIdx.x & 31;
    const bool left_own = lane == 0 || x0 == 0;
    const bool right_own = lane == 31 || x0 + V == (int)pitch;
    RowLoad<S, V, I> ld;
    load_row_flat<S, V, I, POL>(ld, src, links, x0, y, nx, ny, pitch, plane, periodic, left_own, right_own);
    const S *mine = src + ld.r0 + x0;
    using T = typename RowLoad<S, V, I>::T;
    auto own = [&](int q) { return ld_one<POL>(reinterpret_cast<const T *>(mine + q * plane)); };
    finish_row<S, V, FORCE, I, POL>(ld, own, dst, x0, nx, plane, periodic, prm, 0, ld.e, ld.er, left_own, right_own,
                                  active);
}

}  // namespace d2q9
}  // namespace lbm
