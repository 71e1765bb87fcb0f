// D2Q9 device building blocks shared by the single-domain and the batched kernels.
//
// Storage space.  Population q is stored as h_q = s (f_q - w_q) / w_q, s = 1024 for FP16 storage
// and 1 otherwise.  The deviations f_q - w_q of all nine populations scale with w_q, so dividing by
// w_q puts them in one range; the factor 1024 keeps FP16 values out of its subnormal range down to
// deviations of ~1e-7 w_q.  The collision works directly on h: the weights fold into the moment
// sums and drop out of the equilibrium, the forcing term and the moving-wall term, so a stored
// value needs no multiply on the way in or out.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "lbm_internal.h"

namespace lbm {
namespace d2q9 {

// population order: 0:(0,0) 1:(1,0) 2:(0,1) 3:(-1,0) 4:(0,-1) 5:(1,1) 6:(-1,1) 7:(-1,-1) 8:(1,-1)
__host__ __device__ constexpr int cx(int q) { return q == 1 || q == 5 || q == 8 ? 1 : (q == 3 || q == 6 || q == 7 ? -1 : 0); }
__host__ __device__ constexpr int cy(int q) { return q == 2 || q == 5 || q == 6 ? 1 : (q == 4 || q == 7 || q == 8 ? -1 : 0); }
__host__ __device__ constexpr int opp(int q) { return q == 0 ? 0 : (q < 5 ? ((q + 1) & 3) + 1 : ((q - 3) & 3) + 5); }
template <class R>
__host__ __device__ constexpr R w(int q) {
    return q == 0 ? (R)(4.0 / 9.0) : (q < 5 ? (R)(1.0 / 9.0) : (R)(1.0 / 36.0));
}

static_assert(opp(1) == 3 && opp(2) == 4 && opp(3) == 1 && opp(4) == 2, "opp faces");
static_assert(opp(5) == 7 && opp(6) == 8 && opp(7) == 5 && opp(8) == 6, "opp diagonals");

template <class R>
struct Vec2 {
    R x, y;
};

// Arithmetic of the collision with explicit IEEE rounding: these intrinsics are never contracted,
// fused or re-associated by the compiler, so a cell's update is bit-identical in every launch shape
// and in the batched kernel, whatever instruction selection each inlining context gets.
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float mul_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_(double a, double b) { return __dsub_rn(a, b); }

// Two cells at once on the packed FP32 pipe of sm_100+ (FFMA2 / FADD2 / FMUL2): every lane gets the
// same IEEE round-to-nearest result as the scalar intrinsic, so a packed update is bit-identical to
// two scalar ones while issuing half the arithmetic instructions.
__device__ __forceinline__ float2 fma_(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul_(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add_(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b as a + b * (-1): the product is exact, so the one rounding gives a - b (a packed negation
// would cost an instruction of its own)
__device__ __forceinline__ float2 sub_(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

// lane type of an arithmetic type, and a uniform value broadcast to every lane
template <class T>
struct Lane {
    using R = T;
    static __device__ __forceinline__ T bc(R c) { return c; }
};
template <>
struct Lane<float2> {
    using R = float;
    static __device__ __forceinline__ float2 bc(float c) { return make_float2(c, c); }
};

// storage traits: S is the stored type, R the arithmetic type; `to` / `from` convert raw values
template <class S>
struct Store;
template <>
struct Store<float> {
    using R = float;
    static __device__ __forceinline__ R to(float v) { return v; }
    static __device__ __forceinline__ float from(R v) { return v; }
};
template <>
struct Store<double> {
    using R = double;
    static __device__ __forceinline__ R to(double v) { return v; }
    static __device__ __forceinline__ double from(R v) { return v; }
};
template <>
struct Store<__half> {
    using R = float;
    static __device__ __forceinline__ R to(__half v) { return __half2float(v); }
    static __device__ __forceinline__ __half from(R v) { return __float2half_rn(v); }
};
template <>
struct Store<__nv_bfloat16> {
    using R = float;
    static __device__ __forceinline__ R to(__nv_bfloat16 v) { return __bfloat162float(v); }
    static __device__ __forceinline__ __nv_bfloat16 from(R v) { return __float2bfloat16_rn(v); }
};

// s of the storage space
template <class S, class R>
__host__ __device__ constexpr R hscale() {
    return std::is_same<S, __half>::value ? (R)1024 : (R)1;
}

// raw stored value h (read-only path) and back
template <class S>
__device__ __forceinline__ typename Store<S>::R ldh(const S *p) {
    return Store<S>::to(__ldg(p));
}
template <class S>
__device__ __forceinline__ void sth(S *p, typename Store<S>::R v) {
    *p = Store<S>::from(v);
}
// population q as f_q - w_q (host-layout conversion, moments, sums, initialisation)
template <class S>
__device__ __forceinline__ typename Store<S>::R ldq(const S *p, int q) {
    using R = typename Store<S>::R;
    return ldh<S>(p) * (w<R>(q) / hscale<S, R>());
}
template <class S>
__device__ __forceinline__ void stq(S *p, int q, typename Store<S>::R g) {
    using R = typename Store<S>::R;
    sth<S>(p, g * (hscale<S, R>() / w<R>(q)));
}

// V consecutive stored values moved as one 4-, 8- or 16-byte access (p aligned to V*sizeof(S))
template <int B>
struct RawPack;
template <>
struct RawPack<4> {
    using T = unsigned int;
};
template <>
struct RawPack<8> {
    using T = uint2;
};
template <>
struct RawPack<16> {
    using T = uint4;
};

// Two 16-bit values converted together (packed conversions, the same values as one at a time)
template <class S>
struct Pair;
template <>
struct Pair<__half> {
    using P = __half2;
    static __device__ __forceinline__ float2 to(P v) { return __half22float2(v); }
    static __device__ __forceinline__ P from(float a, float b) { return __floats2half2_rn(a, b); }
};
template <>
struct Pair<__nv_bfloat16> {
    using P = __nv_bfloat162;
    static __device__ __forceinline__ float2 to(P v) { return __bfloat1622float2(v); }
    static __device__ __forceinline__ P from(float a, float b) { return __floats2bfloat162_rn(a, b); }
};

// raw V-element pack -> arithmetic values, and back
template <class S, int V, class T>
__device__ __forceinline__ void unpack(const T &raw, typename Store<S>::R (&out)[V]) {
    if constexpr (sizeof(S) == 2 && V % 2 == 0) {
        typename Pair<S>::P e[V / 2];
        memcpy(e, &raw, sizeof(raw));
#pragma unroll
        for (int k = 0; k < V / 2; ++k) {
            const float2 f = Pair<S>::to(e[k]);
            out[2 * k] = f.x;
            out[2 * k + 1] = f.y;
        }
    } else {
        S e[V];
        memcpy(e, &raw, sizeof(raw));
#pragma unroll
        for (int k = 0; k < V; ++k) out[k] = Store<S>::to(e[k]);
    }
}
template <class S, int V, class T>
__device__ __forceinline__ void pack(const typename Store<S>::R (&in)[V], T &raw) {
    if constexpr (sizeof(S) == 2 && V % 2 == 0) {
        typename Pair<S>::P e[V / 2];
#pragma unroll
        for (int k = 0; k < V / 2; ++k) e[k] = Pair<S>::from(in[2 * k], in[2 * k + 1]);
        memcpy(&raw, e, sizeof(raw));
    } else {
        S e[V];
#pragma unroll
        for (int k = 0; k < V; ++k) e[k] = Store<S>::from(in[k]);
        memcpy(&raw, e, sizeof(raw));
    }
}

template <class S, int V>
__device__ __forceinline__ void st_pack(S *__restrict__ p, const typename Store<S>::R (&in)[V]) {
    using T = typename RawPack<sizeof(S) * V>::T;
    T raw;
    pack<S, V>(in, raw);
    *reinterpret_cast<T *>(p) = raw;
}

// L2 eviction-priority policies (PTX createpolicy) for the wide loads and stores of the step:
//   POL 0  no hint
//   POL 1  loads evict_first, stores evict_last: a step's reads are dead once consumed, its writes
//          are the next (reversed) sweep's first reads, so the written half is kept in L2
//   POL 2  loads evict_first, stores without hint
__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

template <class T>
__device__ __forceinline__ T ld_hint(const T *p, uint64_t pol);
template <>
__device__ __forceinline__ uint4 ld_hint<uint4>(const uint4 *p, uint64_t pol) {
    uint4 r;
    asm volatile("ld.global.nc.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "l"(p), "l"(pol));
    return r;
}
template <>
__device__ __forceinline__ uint2 ld_hint<uint2>(const uint2 *p, uint64_t pol) {
    uint2 r;
    asm volatile("ld.global.nc.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;" : "=r"(r.x), "=r"(r.y) : "l"(p), "l"(pol));
    return r;
}
template <>
__device__ __forceinline__ unsigned int ld_hint<unsigned int>(const unsigned int *p, uint64_t pol) {
    unsigned int r;
    asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
    return r;
}
__device__ __forceinline__ void st_hint(uint4 *p, uint4 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z),
                 "r"(v.w), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void st_hint(uint2 *p, uint2 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v2.u32 [%0], {%1, %2}, %3;" ::"l"(p), "r"(v.x), "r"(v.y), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_hint(unsigned int *p, unsigned int v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}

template <class T, int POL>
__device__ __forceinline__ void st_raw_pol(T *__restrict__ p, const T &raw, uint64_t pol) {
    if constexpr (POL != 1)
        *p = raw;
    else
        st_hint(p, raw, pol);
}

template <class S, int V, int POL>
__device__ __forceinline__ void st_pack_pol(S *__restrict__ p, const typename Store<S>::R (&in)[V], uint64_t pol) {
    if constexpr (POL != 1) {
        st_pack<S, V>(p, in);
    } else {
        using T = typename RawPack<sizeof(S) * V>::T;
        T raw;
        pack<S, V>(in, raw);
        st_hint(reinterpret_cast<T *>(p), raw, pol);
    }
}

template <int V>
__device__ __forceinline__ void ld_links(const uint16_t *__restrict__ p, uint32_t (&L)[V]) {
    using T = typename RawPack<2 * V < 4 ? 4 : 2 * V>::T;
    if constexpr (V == 1) {
        L[0] = __ldg(p);
    } else {
        const T raw = __ldg(reinterpret_cast<const T *>(p));
        uint16_t e[V];
        memcpy(e, &raw, sizeof(e));
#pragma unroll
        for (int k = 0; k < V; ++k) L[k] = e[k];
    }
}

template <class R, class P>
__device__ __forceinline__ R omega(const P &p);
template <>
__device__ __forceinline__ float omega<float>(const lbm::D2Q9Params &p) { return p.omega; }
template <>
__device__ __forceinline__ double omega<double>(const lbm::D2Q9Params &p) { return p.omega_d; }
template <class R, class P>
__device__ __forceinline__ Vec2<R> force(const P &p);
template <>
__device__ __forceinline__ Vec2<float> force<float>(const lbm::D2Q9Params &p) { return {p.fx, p.fy}; }
template <>
__device__ __forceinline__ Vec2<double> force<double>(const lbm::D2Q9Params &p) { return {p.fx_d, p.fy_d}; }
template <class R, class P>
__device__ __forceinline__ Vec2<R> wall_u(const P &p);
template <>
__device__ __forceinline__ Vec2<float> wall_u<float>(const lbm::D2Q9Params &p) { return {p.uwx, p.uwy}; }
template <>
__device__ __forceinline__ Vec2<double> wall_u<double>(const lbm::D2Q9Params &p) { return {p.uwx_d, p.uwy_d}; }

// moving-wall term of population q in storage space: s * 6 (c_q . u_w) (the w_q of
// 6 w_q (c_q . u_w) cancels against the 1/w_q of the storage space)
template <class S, class R>
__device__ __forceinline__ R wall_term(int q, Vec2<R> uw) {
    const R cu = cx(q) == 0 ? mul_((R)cy(q), uw.y) : (cy(q) == 0 ? mul_((R)cx(q), uw.x)
                                                             : fma_((R)cx(q), uw.x, mul_((R)cy(q), uw.y)));
    return mul_(hscale<S, R>() * (R)6, cu);
}

// Streamed populations of fluid cell (x, y) in storage space: population q is pulled from
// (x - cx_q, y - cy_q) (periodic wrap, or clamped when the link bit says the value is not used),
// and replaced by the half-way bounce-back of the cell's own opposite population when link bit
// q-1 is set, plus the moving-wall term when bit q+7 is set.
template <class S, class R>
__device__ __forceinline__ void gather(const S *__restrict__ src, uint32_t L, int x, int y, int nx, int ny,
                                       int64_t pitch, int64_t plane, int periodic, Vec2<R> uw, R h[9]) {
    int xm = x - 1, xp = x + 1, ym = y - 1, yp = y + 1;
    if (xm < 0) xm = (periodic & 1) ? nx - 1 : 0;
    if (xp >= nx) xp = (periodic & 1) ? 0 : nx - 1;
    if (ym < 0) ym = (periodic & 2) ? ny - 1 : 0;
    if (yp >= ny) yp = (periodic & 2) ? 0 : ny - 1;
    const int64_t r0 = (int64_t)y * pitch, rm = (int64_t)ym * pitch, rp = (int64_t)yp * pitch;
    h[0] = ldh<S>(src + r0 + x);
    h[1] = ldh<S>(src + 1 * plane + r0 + xm);
    h[2] = ldh<S>(src + 2 * plane + rm + x);
    h[3] = ldh<S>(src + 3 * plane + r0 + xp);
    h[4] = ldh<S>(src + 4 * plane + rp + x);
    h[5] = ldh<S>(src + 5 * plane + rm + xm);
    h[6] = ldh<S>(src + 6 * plane + rm + xp);
    h[7] = ldh<S>(src + 7 * plane + rp + xp);
    h[8] = ldh<S>(src + 8 * plane + rp + xm);
    if (L) {
#pragma unroll
        for (int q = 1; q < 9; ++q) {
            if (L & (1u << (q - 1))) {
                R v = ldh<S>(src + opp(q) * plane + r0 + x);
                if (L & (1u << (q + 7))) v = add_(v, wall_term<S, R>(q, uw));
                h[q] = v;
            }
        }
    }
}

// density deviation and momentum of populations in storage space
template <class S, class T>
__device__ __forceinline__ void moments(const T h[9], T &drho, T &mx, T &my) {
    using R = typename Lane<T>::R;
    constexpr R s = hscale<S, R>();
    const T w0 = Lane<T>::bc(w<R>(0) / s), ws = Lane<T>::bc(w<R>(1) / s), wd = Lane<T>::bc(w<R>(5) / s);
    const T sf = add_(add_(h[1], h[3]), add_(h[2], h[4]));
    const T sd = add_(add_(h[5], h[7]), add_(h[6], h[8]));
    drho = fma_(wd, sd, fma_(ws, sf, mul_(w0, h[0])));
    const T d57 = sub_(h[5], h[7]), d86 = sub_(h[8], h[6]);
    mx = fma_(wd, add_(d57, d86), mul_(ws, sub_(h[1], h[3])));
    my = fma_(wd, sub_(d57, d86), mul_(ws, sub_(h[2], h[4])));
}

// 1/rho: fast FP32 division (__fdividef, within 2 ulp; rho is close to 1), exact division in FP64
template <class R>
__device__ __forceinline__ R recip(R rho) {
    if constexpr (std::is_same<R, float>::value)
        return __fdividef(1.0f, rho);
    else if constexpr (std::is_same<R, float2>::value)
        return make_float2(__fdividef(1.0f, rho.x), __fdividef(1.0f, rho.y));
    else
        return __ddiv_rn(1.0, rho);
}

// shifted equilibrium (f^eq_q - w_q) of (rho, u), in storage space
template <class S, class R>
__device__ __forceinline__ void equilibrium_h(R drho, R rho, R ux, R uy, R h[9]) {
    constexpr R s = hscale<S, R>();
    const R usq = mul_((R)1.5, fma_(ux, ux, mul_(uy, uy)));
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const R cu = fma_((R)cx(q), ux, mul_((R)cy(q), uy));
        const R t = sub_(fma_(mul_((R)4.5, cu), cu, mul_((R)3, cu)), usq);
        h[q] = mul_(s, fma_(rho, t, drho));
    }
}

template <class S>
struct is_half_store : std::false_type {};
template <>
struct is_half_store<__half> : std::true_type {};
template <>
struct is_half_store<__nv_bfloat16> : std::true_type {};

// Conservative rounding for 16-bit storage.  Rounding the nine post-collision populations to FP16
// or BF16 one by one leaves residuals in mass and momentum that are conserved by the dynamics and
// so accumulate step after step (and a body-force increment smaller than half an ulp is lost every
// step).  Here the rounding residuals r_q = h_q - round(h_q) of the rest and axis populations are
// moved into the diagonal populations before those are rounded: in f space the residual mass and
// momentum are spread over the four diagonals as a_d = (dm + c_d . dj) / 4, which in storage space
// (h = s f / w, w_0 = 16 w_d, w_axis = 4 w_d) is  h_d += 4 r_0 + 2 (r_a + r_b)  with a, b the axis
// populations with c_a + c_b = c_d.  What remains is the diagonals' own rounding, whose absolute
// resolution is 4x (momentum) and 16x (mass) finer.
// With `packed` (float2 only), the stored pairs of populations 0-4 are also returned: packing the
// rounded values again would give the same words.
template <class S, class T>
__device__ __forceinline__ void conserve_rounding(T h[9], uint32_t *packed = nullptr) {
    T r[5];
    if constexpr (std::is_same<T, float2>::value) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {  // the two cells' values of population q round-trip together
            const typename Pair<S>::P p = Pair<S>::from(h[q].x, h[q].y);
            if (packed) memcpy(&packed[q], &p, sizeof(p));
            const float2 hr = Pair<S>::to(p);
            r[q] = sub_(h[q], hr);
            h[q] = hr;
        }
    } else {
#pragma unroll
        for (int q = 0; q < 4; q += 2) {  // round trips two at a time
            const float2 hr = Pair<S>::to(Pair<S>::from(h[q], h[q + 1]));
            r[q] = sub_(h[q], hr.x);
            r[q + 1] = sub_(h[q + 1], hr.y);
            h[q] = hr.x;
            h[q + 1] = hr.y;
        }
        const T hr = Store<S>::to(Store<S>::from(h[4]));
        r[4] = sub_(h[4], hr);
        h[4] = hr;
    }
    const T two = Lane<T>::bc(2), r0x4 = mul_(Lane<T>::bc(4), r[0]);
    h[5] = add_(h[5], fma_(two, add_(r[1], r[2]), r0x4));
    h[6] = add_(h[6], fma_(two, add_(r[2], r[3]), r0x4));
    h[7] = add_(h[7], fma_(two, add_(r[3], r[4]), r0x4));
    h[8] = add_(h[8], fma_(two, add_(r[4], r[1]), r0x4));
}

// BGK collision with Guo forcing, in place, in storage space.  Opposite populations q, q' share
// c_q . u with opposite signs, so the equilibrium and the forcing term split into a symmetric part
// A and an antisymmetric part B per pair: h_q <- (1 - om) h_q + A + B, h_q' <- (1 - om) h_q' + A - B,
//   A = om s (drho + rho (4.5 cu^2 - 1.5 u^2)) + s (1 - om/2) (9 cu cF - 3 u.F)
//   B = 3 om s rho cu + 3 s (1 - om/2) cF
// T is the scalar arithmetic type R, or float2 for two cells at once (uniform quantities -- omega,
// the force and what depends only on them -- are computed in R and broadcast, which gives every
// lane the scalar path's values).
template <class S, class T, bool FORCE>
__device__ __forceinline__ void collide_t(T h[9], typename Lane<T>::R om, Vec2<typename Lane<T>::R> F,
                                          uint32_t *packed = nullptr) {
    using R = typename Lane<T>::R;
    auto B = [](R c) { return Lane<T>::bc(c); };
    constexpr R s = hscale<S, R>();
    T drho, mx, my;
    moments<S, T>(h, drho, mx, my);
    const T rho = add_(B((R)1), drho);
    const T inv = recip(rho);
    T ux, uy;
    if (FORCE) {
        ux = mul_(fma_(B((R)0.5), B(F.x), mx), inv);
        uy = mul_(fma_(B((R)0.5), B(F.y), my), inv);
    } else {
        ux = mul_(mx, inv);
        uy = mul_(my, inv);
    }
    // -1.5 u^2 (negated products are exact, so every expression below equals the one with the
    // negation written out)
    const T nusq = mul_(B((R)-1.5), fma_(ux, ux, mul_(uy, uy)));
    const T om1 = B(sub_((R)1, om));
    const T omv = B(om);
    const T om_s_drho = mul_(omv, mul_(B(s), drho));
    const T om_s_rho = mul_(omv, mul_(B(s), rho));
    const T om_s_rho3 = mul_(B((R)3), om_s_rho);
    R pre = 0, pre3 = 0;
    T nuF3 = B((R)0);  // -3 u.F
    if (FORCE) {
        pre = mul_(s, fma_((R)-0.5, om, (R)1));
        pre3 = mul_((R)3, pre);
        nuF3 = mul_(B((R)-3), fma_(ux, B(F.x), mul_(uy, B(F.y))));
    }
    // rest population: h0eq = s (drho - rho usq), forcing s (1 - om/2) (-3 u.F)
    {
        T a = fma_(om_s_rho, nusq, om_s_drho);
        if (FORCE) a = fma_(B(pre), nuF3, a);
        h[0] = fma_(om1, h[0], a);
    }
    auto pair = [&](int q, int qb, T cu, R cF) {
        T a = fma_(om_s_rho, fma_(mul_(B((R)4.5), cu), cu, nusq), om_s_drho);
        T b = mul_(om_s_rho3, cu);
        if (FORCE) {
            a = fma_(B(pre), fma_(mul_(B((R)9), cu), B(cF), nuF3), a);
            b = fma_(B(pre3), B(cF), b);
        }
        h[q] = fma_(om1, h[q], add_(a, b));
        h[qb] = fma_(om1, h[qb], sub_(a, b));
    };
    pair(1, 3, ux, F.x);
    pair(2, 4, uy, F.y);
    pair(5, 7, add_(ux, uy), add_(F.x, F.y));
    pair(8, 6, sub_(ux, uy), sub_(F.x, F.y));
    if constexpr (is_half_store<S>::value) conserve_rounding<S, T>(h, packed);
}

template <class S, class R, bool FORCE>
__device__ __forceinline__ void collide(R h[9], R om, Vec2<R> F) {
    collide_t<S, R, FORCE>(h, om, F);
}

}  // namespace d2q9
}  // namespace lbm
