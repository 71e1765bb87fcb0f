// D3Q27_REF kernels: the reference's step (simulation/source/SimCalcFuncs.cu) re-designed as
// structure-of-arrays passes.
//
// State: f[q * cells + cell], q in the reference's particle_distribution order, cell index
// z + Z*(y + Y*x) (Lattice.cpp:254).  FP32 populations; the equilibrium is evaluated in FP64 and
// rounded to FP32, as the reference's double literals make it (SimCalcFuncs.cu:125-154).
//
// The reference runs four kernels per CLI step with a full-lattice malloc + device copy before the
// streaming and reflection kernels (Lattice.cpp:115-210) and float atomics on every population.
// Here one step is one pass over the populations (one read, one write):
//   fused_kernel   all cells that receive no reflection: zero-fill pull streaming, zeroing of
//                  internal cells, collision, flow source.
//   gather_kernel  the (few) fluid cells next to reflecting cells: the same, plus the reflected
//                  populations pulled through precomputed gather lists (the reference's atomic
//                  scatter of SimCalcFuncs.cu:164-186 turned into a pull with a fixed order), plus
//                  the momentum-exchange force reduced per block without atomics.
// lbm_apply() runs the reference's single passes (stream / reflect / collide / flow) separately.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>

#include "lbm_internal.h"
#include "pdl.cuh"
#include "reduce.cuh"

namespace lbm {
namespace {

constexpr uint8_t F_INTERNAL = LBM_INTERNAL, F_SOURCE = LBM_SOURCE;
constexpr uint8_t F_GATHER = 8;  // cell receives reflected populations (set by the library)

// SimCalcFuncs.cu:12-14
__constant__ int c_dir[27][3] = {
    {0, 0, 0},   {-1, 0, 0},  {0, -1, 0},  {0, 0, -1},  {0, 0, 1},    {0, 1, 0},    {1, 0, 0},
    {-1, -1, 0}, {-1, 0, -1}, {-1, 0, 1},  {-1, 1, 0},  {0, -1, -1},  {0, -1, 1},   {0, 1, -1},
    {0, 1, 1},   {1, -1, 0},  {1, 0, -1},  {1, 0, 1},   {1, 1, 0},    {-1, -1, -1}, {-1, -1, 1},
    {-1, 1, -1}, {-1, 1, 1},  {1, -1, -1}, {1, -1, 1},  {1, 1, -1},   {1, 1, 1}};
__constant__ float c_split[27] = {0.0f,        1.0f,        1.0f,        1.0f,        1.0f,        1.0f,
                                  1.0f,        0.5f,        0.5f,        0.5f,        0.5f,        0.5f,
                                  0.5f,        0.5f,        0.5f,        0.5f,        0.5f,        0.5f,
                                  0.5f,        1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 3.0f,
                                  1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 3.0f};

// Unsigned 32-bit division by an invariant divisor with one multiply-high, two shifts and two adds
// (Granlund and Montgomery, "Division by invariant integers using multiplication", PLDI 1994,
// section 4): with l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1,
// n / d = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0), t = mulhi(m, n), for every 32-bit n.
struct FastDiv {
    uint32_t d, m;
    int s1, s2;
    static FastDiv make(uint32_t d) {
        int l = 0;
        while (l < 32 && (1ull << l) < d) ++l;
        FastDiv f;
        f.d = d;
        f.m = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
        f.s1 = l < 1 ? l : 1;
        f.s2 = l > 1 ? l - 1 : 0;
        return f;
    }
    __device__ __forceinline__ uint32_t div(uint32_t n) const {
        const uint32_t t = __umulhi(m, n);
        return (t + ((n - t) >> s1)) >> s2;
    }
};

// The same tables as compile-time functions, for loops that are unrolled over the 27 directions:
// every direction-dependent operand folds to an immediate (products by 0 vanish, by +-1 become
// additions or subtractions).
__host__ __device__ constexpr int kd(int j, int a) {
    constexpr int t[27][3] = {
        {0, 0, 0},   {-1, 0, 0},  {0, -1, 0},  {0, 0, -1},  {0, 0, 1},    {0, 1, 0},    {1, 0, 0},
        {-1, -1, 0}, {-1, 0, -1}, {-1, 0, 1},  {-1, 1, 0},  {0, -1, -1},  {0, -1, 1},   {0, 1, -1},
        {0, 1, 1},   {1, -1, 0},  {1, 0, -1},  {1, 0, 1},   {1, 1, 0},    {-1, -1, -1}, {-1, -1, 1},
        {-1, 1, -1}, {-1, 1, 1},  {1, -1, -1}, {1, -1, 1},  {1, 1, -1},   {1, 1, 1}};
    return t[j][a];
}
__host__ __device__ constexpr int opp27(int j) {
    int r = 0;
    for (int p = 0; p < 27; ++p)
        if (kd(p, 0) == -kd(j, 0) && kd(p, 1) == -kd(j, 1) && kd(p, 2) == -kd(j, 2)) r = p;
    return r;
}
__host__ __device__ constexpr float ks(int j) { return j == 0 ? 0.0f : (j < 7 ? 1.0f : (j < 19 ? 0.5f : 1.0f / 3.0f)); }

// c_j . u = ((c_jx ux) + (c_jy uy)) + (c_jz uz) with the zero terms left out: the products by
// -1, 0, 1 are exact and adding an exact zero changes no non-zero value, so this is the
// reference's FP32 value (up to the sign of a zero result)
template <int J>
__device__ __forceinline__ float cdot(float ux, float uy, float uz) {
    float s = 0.0f;
    bool any = false;
    const float u[3] = {ux, uy, uz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (kd(J, a) == 0) continue;
        const float t = kd(J, a) > 0 ? u[a] : -u[a];
        s = any ? __fadd_rn(s, t) : t;
        any = true;
    }
    return s;
}

// SPLIT-weighted first moment (SimCalcFuncs.cu:109-113): m_a += f_j c_ja SPLIT_j over j, the zero
// terms left out (an exact zero added to the running sum changes nothing for finite populations).
// Each term is one fused multiply-add, m_a = RN((f_j c_ja) SPLIT_j + m_a) (f_j c_ja is exact), written
// with the explicit intrinsic so that every kernel rounds it the same way.
template <int J>
__device__ __forceinline__ void split_moment(float v, float &mx, float &my, float &mz) {
    if (kd(J, 0)) mx = __fmaf_rn(kd(J, 0) > 0 ? v : -v, ks(J), mx);
    if (kd(J, 1)) my = __fmaf_rn(kd(J, 1) > 0 ? v : -v, ks(J), my);
    if (kd(J, 2)) mz = __fmaf_rn(kd(J, 2) > 0 ? v : -v, ks(J), mz);
}

// |u|^2 = (ux ux + uy uy) + uz uz as two fused multiply-adds, the same in every kernel
__device__ __forceinline__ float usq_of(float ux, float uy, float uz) {
    return __fmaf_rn(uz, uz, __fmaf_rn(uy, uy, __fmul_rn(ux, ux)));
}

template <int J>
struct Unroll {
    template <class F>
    static __device__ __forceinline__ void run(F &&f) {
        Unroll<J - 1>::run(f);
        f(std::integral_constant<int, J - 1>{});
    }
};
template <>
struct Unroll<0> {
    template <class F>
    static __device__ __forceinline__ void run(F &&) {}
};

struct Dims {
    int X, Y, Z;
    int64_t n;
    FastDiv dz, dy;  // division by Z and by Y
};

// cell index -> (x, y, z); cells < 2^31, so the index fits 32 bits
__device__ __forceinline__ void decode(const Dims &d, int64_t c, int &x, int &y, int &z) {
    const uint32_t u = (uint32_t)c;
    const uint32_t t = d.dz.div(u);
    z = (int)(u - t * (uint32_t)d.Z);
    const uint32_t xq = d.dy.div(t);
    y = (int)(t - xq * (uint32_t)d.Y);
    x = (int)xq;
}

// pull streaming with zero fill (SimCalcFuncs.cu:79-96): v[j] = f_j(x - c_j), 0 outside
__device__ __forceinline__ void pull(const float *__restrict__ src, const Dims &d, int64_t c, int x, int y, int z,
                                     float v[27]) {
    if (x > 0 && y > 0 && x < d.X - 1 && y < d.Y - 1) {
        // every x and y neighbour exists (uniform over a block when Z is a multiple of the block
        // size: its cells are then one column of z); a neighbour beyond the first or last z is
        // zero, its load predicated off, so a warp holding z = 0 or z = Z - 1 does not diverge
        const int64_t sy = d.Z, sx = (int64_t)d.Z * d.Y;
        const bool zlo = z > 0, zhi = z < d.Z - 1;
        Unroll<27>::run([&](auto jj) {
            constexpr int j = decltype(jj)::value;
            int64_t s = c - kd(j, 2);
            if (kd(j, 1)) s = kd(j, 1) > 0 ? s - sy : s + sy;
            if (kd(j, 0)) s = kd(j, 0) > 0 ? s - sx : s + sx;
            if constexpr (kd(j, 2) == 0)
                v[j] = __ldg(src + (int64_t)j * d.n + s);
            else
                v[j] = (kd(j, 2) > 0 ? zlo : zhi) ? __ldg(src + (int64_t)j * d.n + s) : 0.0f;
        });
        return;
    }
#pragma unroll
    for (int j = 0; j < 27; ++j) {
        const int sx = x - c_dir[j][0], sy = y - c_dir[j][1], sz = z - c_dir[j][2];
        const bool in = sx >= 0 && sy >= 0 && sz >= 0 && sx < d.X && sy < d.Y && sz < d.Z;
        // neighbours outside the lattice are never addressed: their index is replaced by the cell's own
        const int64_t s = in ? c - (int64_t)c_dir[j][2] - (int64_t)d.Z * ((int64_t)c_dir[j][1] + (int64_t)d.Y * c_dir[j][0]) : c;
        v[j] = in ? __ldg(src + (int64_t)j * d.n + s) : 0.0f;
    }
}

// ------------------------------------------------------------------------- equilibrium
// The reference evaluates eq_i = W_i * rho * (1 + 3 ct + 4.5 ct^2 - 1.5 usq) in FP64 from FP32 ct,
// usq and rho, and rounds it to FP32 (SimCalcFuncs.cu:122-155).  3 ct, 4.5 ct * ct and 1.5 usq
// are exact in FP64, so that value is E = fl64(fl64(W rho) * fl64(fl64(fl64(1 + A) + B) - C)),
// whichever way the compiler contracts the expression.  GB300 runs FP64 at a small fraction of its
// FP32 rate, which made the FP64 pipe the bound of this step.  eq_fast() evaluates E in float-float
// arithmetic (error-free two-sum / FMA two-product transformations, Dekker 1971, Knuth TAOCP 4.2.2)
// to within 2^-42 * |W rho| * (1 + |A| + B + C) of the FP64 value, rounds it to FP32, and accepts
// the result only when that error bound keeps the FP64 value strictly inside the same FP32 rounding
// interval; otherwise (about one evaluation in 10^5) it evaluates the FP64 expression itself.
// Either way the result is the reference's FP64-evaluated equilibrium, bit for bit.
// the four weights (SimCalcFuncs.cu:126,135,144,153) in FP64, and split into FP32 hi + lo
__host__ __device__ constexpr double kW(int k) {
    return k == 0 ? 8.0 / 27.0 : (k == 1 ? 2.0 / 27.0 : (k == 2 ? 1.0 / 54.0 : 1.0 / 216.0));
}
__host__ __device__ constexpr float kWhi(int k) { return (float)kW(k); }
__host__ __device__ constexpr float kWlo(int k) { return (float)(kW(k) - (double)(float)kW(k)); }
__host__ __device__ constexpr int wclass(int i) { return i == 0 ? 0 : (i < 7 ? 1 : (i < 19 ? 2 : 3)); }
// the n-th direction i (0 < i < opposite(i)) that stands for a pair of opposite directions (13 pairs)
__host__ __device__ constexpr int pair_rep(int n) {
    for (int i = 1; i < 27; ++i)
        if (i < opp27(i) && n-- == 0) return i;
    return -1;
}

// The float-float helpers are written once for T = float and T = float2: a float2 carries two
// independent evaluations (two pairs of directions) through the paired FP32 instructions of sm_100+
// (__fadd2_rn, __fmul2_rn, __ffma2_rn), whose every lane rounds as the scalar instruction, so both
// forms give the same bits.  a - b is a + (-b), the same IEEE value.
__device__ __forceinline__ float ff_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float ff_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float ff_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float ff_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float ff_neg(float a) { return -a; }
__device__ __forceinline__ float ff_abs(float a) { return fabsf(a); }
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 ff_sub(float2 a, float2 b) { return __fadd2_rn(a, ff_neg(b)); }
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 ff_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 ff_abs(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
template <class T>
__device__ __forceinline__ T ff_bc(float c);
template <>
__device__ __forceinline__ float ff_bc<float>(float c) { return c; }
template <>
__device__ __forceinline__ float2 ff_bc<float2>(float c) { return make_float2(c, c); }

// per-lane flags of T
struct Ok2 {
    bool x, y;
};
template <class T>
struct OkOf {
    using type = bool;
};
template <>
struct OkOf<float2> {
    using type = Ok2;
};

// s + e == a + b exactly
template <class T>
__device__ __forceinline__ void two_sum(T a, T b, T &s, T &e) {
    s = ff_add(a, b);
    const T bv = ff_sub(s, a);
    const T av = ff_sub(s, bv);
    e = ff_add(ff_sub(a, av), ff_sub(b, bv));
}

// the reference's expression, FP64 (the fallback and the LBM_EQ_FP64 path)
__device__ __forceinline__ float eq_fp64(int k, float density, float ct, float usq) {
    return (float)(kW(k) * density * (1 + (3.0 * ct) + (4.5 * ct * ct) - (1.5 * usq)));
}

// ph + pl: W_k * rho within 2^-47; c1 + c1e == 1.5 usq exactly.  Returns the FP32 rounding of the
// float-float value; ok says whether it is proven equal to the FP64 evaluation.
// s + e == a + b exactly when |a| >= |b| (Dekker's fast two-sum)
template <class T>
__device__ __forceinline__ void fast_two_sum(T a, T b, T &s, T &e) {
    s = ff_add(a, b);
    e = ff_sub(b, ff_sub(s, a));
}

// accept r when |E_ff - E_fp64| <= t (t = |d| + m rounded up by RN's monotonicity) keeps the FP64
// value strictly inside r's FP32 rounding interval: t below half the smaller gap next to r
// (2^e * 2^-24, or 2^-25 at a power of two), r normal and far from underflow, finite
__device__ __forceinline__ bool ff_accept(float r, float t) {
    const uint32_t rb = __float_as_uint(r) & 0x7fffffffu;
    const uint32_t ex = rb & 0x7f800000u;
    const float half_gap = __fmul_rn(__uint_as_float(ex), (rb & 0x7fffffu) ? 0x1p-24f : 0x1p-25f);
    return ex >= (67u << 23) && ex < 0x7f800000u && t < half_gap;
}
__device__ __forceinline__ void ff_accept(float r, float t, bool &ok) { ok = ff_accept(r, t); }
__device__ __forceinline__ void ff_accept(float2 r, float2 t, Ok2 &ok) {
    ok.x = ff_accept(r.x, t.x);
    ok.y = ff_accept(r.y, t.y);
}

// E = (ph + pl) * (1 + s2 + lo) rounded to FP32, with the acceptance test against the bound m on
// |E_ff - E_fp64| (see above).
template <class T>
__device__ __forceinline__ T ff_finish(T ph, T pl, T m, T s2, T lo, typename OkOf<T>::type &ok) {
    T th, e3;
    two_sum(ff_bc<T>(1.0f), s2, th, e3);
    const T tl = ff_add(e3, lo);                                          // T = th + tl
    const T eh = ff_mul(ph, th);
    const T el = ff_fma(ph, tl, ff_fma(pl, th, ff_fma(ph, th, ff_neg(eh))));
    const T r = ff_add(eh, el);
    const T d = ff_add(ff_sub(eh, r), el);                                // (eh + el) - r
    ff_accept(r, ff_add(ff_abs(d), m), ok);
    return r;
}

__device__ __forceinline__ bool ok_and(bool a, bool b) { return a && b; }
__device__ __forceinline__ Ok2 ok_and(Ok2 a, Ok2 b) { return Ok2{a.x && b.x, a.y && b.y}; }
__device__ __forceinline__ bool ab_ok(float a, float b) { return fabsf(a) >= b; }
__device__ __forceinline__ Ok2 ab_ok(float2 a, float2 b) { return Ok2{fabsf(a.x) >= b.x, fabsf(a.y) >= b.y}; }

// The pair of opposite directions (c . u = ct and -ct) shares ct^2, B and the bound: mk = |ph| 2^-42,
// c1p = 1 + 1.5 usq rounded (M = 1 + |A| + B + C up to rounding, well inside the bound's margin).
template <class T>
__device__ __forceinline__ void eq_ff_pair(T ph, T pl, T mk, T c1, T c1e, T c1p, T ct, T &rp,
                                           typename OkOf<T>::type &okp, T &rn, typename OkOf<T>::type &okn) {
    const T three = ff_bc<T>(3.0f), four5 = ff_bc<T>(4.5f);
    const T a = ff_mul(three, ct), ae = ff_fma(three, ct, ff_neg(a));        // A = 3 ct (for -ct: -a, -ae)
    const T p = ff_mul(ct, ct), pe = ff_fma(ct, ct, ff_neg(p));             // ct^2
    const T b = ff_mul(four5, p), be = ff_fma(four5, p, ff_neg(b));         // B = 4.5 ct^2 = b + be + 4.5 pe
    const T bb = ff_sub(ff_add(be, ff_mul(four5, pe)), c1e);                // low parts of B - C
    const T m = ff_mul(mk, ff_add(ff_add(c1p, ff_abs(a)), b));
    // A + B by the fast two-sum, exact for |A| >= B (|ct| up to about 2/3); otherwise FP64
    const auto ab = ab_ok(a, b);
    T s1, e1, s2, e2;
    fast_two_sum(a, b, s1, e1);
    two_sum(s1, ff_neg(c1), s2, e2);
    rp = ff_finish(ph, pl, m, s2, ff_add(ff_add(ff_add(ae, bb), e1), e2), okp);
    fast_two_sum(ff_neg(a), b, s1, e1);
    two_sum(s1, ff_neg(c1), s2, e2);
    rn = ff_finish(ph, pl, m, s2, ff_add(ff_add(ff_add(ff_neg(ae), bb), e1), e2), okn);
    okp = ok_and(okp, ab);
    okn = ok_and(okn, ab);
}

__device__ __forceinline__ float eq_ff(float ph, float pl, float c1, float c1e, float ct, bool &ok) {
    const float a = __fmul_rn(3.0f, ct), ae = __fmaf_rn(3.0f, ct, -a);      // A = 3 ct
    const float p = __fmul_rn(ct, ct), pe = __fmaf_rn(ct, ct, -p);         // ct^2
    const float b = __fmul_rn(4.5f, p), be = __fmaf_rn(4.5f, p, -b);       // B = 4.5 ct^2 = b + be + 4.5 pe
    float s1, e1, s2, e2, th, e3;
    two_sum(a, b, s1, e1);
    two_sum(s1, -c1, s2, e2);
    const float lo = __fadd_rn(__fadd_rn(__fsub_rn(__fadd_rn(__fadd_rn(ae, be), __fmul_rn(4.5f, pe)), c1e), e1), e2);
    two_sum(1.0f, s2, th, e3);
    const float tl = __fadd_rn(e3, lo);                                   // T = th + tl
    const float eh = __fmul_rn(ph, th);
    const float el = __fmaf_rn(ph, tl, __fmaf_rn(pl, th, __fmaf_rn(ph, th, -eh)));
    const float r = __fadd_rn(eh, el);
    const float d = __fadd_rn(__fsub_rn(eh, r), el);                      // (eh + el) - r
    const float m = __fmul_rn(__fmul_rn(fabsf(ph), __fadd_rn(__fadd_rn(__fadd_rn(1.0f, fabsf(a)), b), c1)), 0x1p-42f);
    ok = ff_accept(r, __fadd_rn(fabsf(d), m));
    return r;
}

// ------------------------------------------------------------------------- division by tau
// The update divides by tau 27 times per cell (SimCalcFuncs.cu:128).  With y = RN(1/tau), the
// quotient q = RN(x y) corrected once, RN(q + RN(x - tau q) y) (Markstein, IBM J. Res. Dev. 34(1),
// 1990), is the correctly rounded x / tau; each tau the library uses is first checked against the
// IEEE division for all 2^32 float inputs (tau_check), and the correction is used only for a tau
// that passes, and only for |x| in [2^-96, 2^96] (elsewhere: the IEEE division).
struct Tau {
    float b;   // tau
    float y;   // RN(1 / tau)
    int fast;  // 1: tau passed the exhaustive check
};

// the corrected reciprocal product where it is the IEEE quotient (ok), for |x| in [2^-96, 2^96] or 0
__device__ __forceinline__ float div_fast(float x, const Tau &t, bool &ok) {
    const float ax = fabsf(x);
    ok = t.fast && ax <= 0x1p96f && (ax >= 0x1p-96f || ax == 0.0f);
    if (ax == 0.0f) return t.b > 0.0f ? x : -x;  // +-0 / tau
    const float q = __fmul_rn(x, t.y);
    return __fmaf_rn(__fmaf_rn(-q, t.b, x), t.y, q);
}

// the same for two values at once (paired instructions; per lane as div_fast)
__device__ __forceinline__ float2 div_fast2(float2 x, const Tau &t, Ok2 &ok) {
    const float2 y = make_float2(t.y, t.y), b = make_float2(t.b, t.b);
    const float2 q = __fmul2_rn(x, y);
    float2 r = __ffma2_rn(__ffma2_rn(ff_neg(q), b, x), y, q);
    const float ax = fabsf(x.x), ay = fabsf(x.y);
    ok.x = t.fast && ax <= 0x1p96f && (ax >= 0x1p-96f || ax == 0.0f);
    ok.y = t.fast && ay <= 0x1p96f && (ay >= 0x1p-96f || ay == 0.0f);
    if (ax == 0.0f) r.x = t.b > 0.0f ? x.x : -x.x;  // +-0 / tau
    if (ay == 0.0f) r.y = t.b > 0.0f ? x.y : -x.y;
    return r;
}

__device__ __forceinline__ float div_tau(float x, const Tau &t) {
    bool ok;
    const float q = div_fast(x, t, ok);
    return ok ? q : __fdiv_rn(x, t.b);
}

__global__ void tau_check_kernel(float b, float *y_out, unsigned long long *bad) {
    const Tau t{b, __frcp_rn(b), 1};
    if (blockIdx.x == 0 && threadIdx.x == 0) *y_out = t.y;
    unsigned long long n = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < (1ull << 32); i += (uint64_t)gridDim.x * blockDim.x) {
        const float x = __uint_as_float((uint32_t)i);
        const float a = div_tau(x, t), e = __fdiv_rn(x, b);
        n += __float_as_uint(a) != __float_as_uint(e) && !(a != a && e != e);
    }
    atomicAdd(bad, n);
}

// calculate_collision (SimCalcFuncs.cu:98-156): FP32 density and SPLIT-weighted velocity, FP64
// equilibrium rounded to FP32, f += (eq - f) / tau in FP32.  EQ64: the FP64 expression for every
// direction.  Otherwise the float-float evaluation; if its bound cannot decide any direction of the
// cell (about one cell in 10^4), the function returns false and leaves v undefined, and the caller
// recomputes the cell with EQ64 -- keeping the FP64 code off the common path.
template <bool EQ64>
__device__ __forceinline__ bool collide(float v[27], const Tau &tau) {
    float density = 0.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f;
    Unroll<27>::run([&](auto ii) {
        constexpr int i = decltype(ii)::value;
        density += v[i];
        split_moment<i>(v[i], ux, uy, uz);
    });
    if (density != 0.0f) {
        ux /= density;
        uy /= density;
        uz /= density;
    }
    const float usq = usq_of(ux, uy, uz);
    if (EQ64) {
        Unroll<27>::run([&](auto ii) {
            constexpr int i = decltype(ii)::value;
            v[i] = v[i] + div_tau(eq_fp64(wclass(i), density, cdot<i>(ux, uy, uz), usq) - v[i], tau);
        });
        return true;
    }
    float ph[4], pl[4], mk[4];
    const float c1 = __fmul_rn(1.5f, usq), c1e = __fmaf_rn(1.5f, usq, -c1), c1p = __fadd_rn(1.0f, c1);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        ph[k] = __fmul_rn(kWhi(k), density);
        pl[k] = __fmaf_rn(kWlo(k), density, __fmaf_rn(kWhi(k), density, -ph[k]));
        mk[k] = __fmul_rn(fabsf(ph[k]), 0x1p-42f);
    }
    // a cell with zero density and velocity (e.g. an internal, zeroed cell): the FP64 value is
    // W * density * 1, a zero with the sign of the density
    const bool still = density == 0.0f && usq == 0.0f;
    const float zero = copysignf(0.0f, density);
    bool all_ok = true;
    // division: the corrected reciprocal product only; an input outside its range (or a tau that
    // failed the check) sends the cell to the FP64 recomputation like an undecided equilibrium
    auto relax = [&](float &f, float eq) {
        bool ok;
        f = f + div_fast(eq - f, tau, ok);
        all_ok = all_ok && ok;
    };
    {
        bool ok;
        const float eq = eq_ff(ph[0], pl[0], c1, c1e, 0.0f, ok);
        all_ok = ok || still;
        relax(v[0], still ? zero : eq);
    }
    // the 13 pairs of opposite directions, two pairs per paired instruction, the last one alone
    auto relax2 = [&](float &f0, float &f1, float2 eq) {
        Ok2 ok;
        const float2 q = div_fast2(__fadd2_rn(eq, make_float2(-f0, -f1)), tau, ok);
        f0 = __fadd_rn(f0, q.x);
        f1 = __fadd_rn(f1, q.y);
        all_ok = all_ok && ok.x && ok.y;
    };
    const float2 c1_2 = make_float2(c1, c1), c1e_2 = make_float2(c1e, c1e), c1p_2 = make_float2(c1p, c1p);
    Unroll<6>::run([&](auto nn) {
        constexpr int n = decltype(nn)::value;
        constexpr int i0 = pair_rep(2 * n), i1 = pair_rep(2 * n + 1);
        constexpr int j0 = opp27(i0), j1 = opp27(i1);
        constexpr int k0 = wclass(i0), k1 = wclass(i1);
        float2 rp, rn;
        Ok2 okp, okn;
        eq_ff_pair(make_float2(ph[k0], ph[k1]), make_float2(pl[k0], pl[k1]), make_float2(mk[k0], mk[k1]), c1_2, c1e_2,
                   c1p_2, make_float2(cdot<i0>(ux, uy, uz), cdot<i1>(ux, uy, uz)), rp, okp, rn, okn);
        all_ok = all_ok && ((okp.x && okn.x && okp.y && okn.y) || still);
        relax2(v[i0], v[i1], still ? make_float2(zero, zero) : rp);
        relax2(v[j0], v[j1], still ? make_float2(zero, zero) : rn);
    });
    {
        constexpr int i = pair_rep(12), j = opp27(i), k = wclass(i);
        float rp, rn;
        bool okp, okn;
        eq_ff_pair(ph[k], pl[k], mk[k], c1, c1e, c1p, cdot<i>(ux, uy, uz), rp, okp, rn, okn);
        all_ok = all_ok && ((okp && okn) || still);
        relax(v[i], still ? zero : rp);
        relax(v[j], still ? zero : rn);
    }
    static_assert(pair_rep(12) > 0 && pair_rep(13) < 0, "13 pairs of opposite directions");
    return all_ok;
}

// calculate_collision with the equilibrium in FP32 (LBM_EQ_FP32): the same FP32 density and
// SPLIT-weighted velocity as above, then eq_i = W_i rho (1 + 3 ct + 4.5 ct^2 - 1.5 usq) in FP32 --
// for a pair of opposite directions W rho ((1 - 1.5 usq) + 4.5 ct^2 +- 3 ct) shares everything but
// the sign of 3 ct -- and f += (eq - f) / tau by the corrected reciprocal product (the IEEE quotient
// for a tau that passed the exhaustive check and |x| in [2^-96, 2^96]; within an ulp elsewhere).
// Against the FP64-evaluated equilibrium of the reference each value differs by a few FP32 ulps, far
// inside a 1e-5 relative tolerance.  Two pairs per paired FP32 instruction.
__device__ __forceinline__ void collide_fp32(float v[27], const Tau &tau) {
    float density = 0.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f;
    Unroll<27>::run([&](auto ii) {
        constexpr int i = decltype(ii)::value;
        density += v[i];
        split_moment<i>(v[i], ux, uy, uz);
    });
    if (density != 0.0f) {
        ux /= density;
        uy /= density;
        uz /= density;
    }
    const float base = __fmaf_rn(-1.5f, usq_of(ux, uy, uz), 1.0f);
    float wr[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) wr[k] = __fmul_rn(kWhi(k), density);
    auto rel = [&](float x) {
        const float q = __fmul_rn(x, tau.y);
        return __fmaf_rn(__fmaf_rn(-q, tau.b, x), tau.y, q);
    };
    v[0] = __fadd_rn(v[0], rel(__fsub_rn(__fmul_rn(wr[0], base), v[0])));
    const float2 y2 = make_float2(tau.y, tau.y), b2 = make_float2(tau.b, tau.b);
    auto rel2 = [&](float2 x) {
        const float2 q = __fmul2_rn(x, y2);
        return __ffma2_rn(__ffma2_rn(make_float2(-q.x, -q.y), b2, x), y2, q);
    };
    const float2 base2 = make_float2(base, base), three = make_float2(3.0f, 3.0f), four5 = make_float2(4.5f, 4.5f);
    Unroll<6>::run([&](auto nn) {
        constexpr int n = decltype(nn)::value;
        constexpr int i0 = pair_rep(2 * n), i1 = pair_rep(2 * n + 1);
        constexpr int j0 = opp27(i0), j1 = opp27(i1);
        const float2 ct = make_float2(cdot<i0>(ux, uy, uz), cdot<i1>(ux, uy, uz));
        const float2 w = make_float2(wr[wclass(i0)], wr[wclass(i1)]);
        const float2 sym = __ffma2_rn(__fmul2_rn(four5, ct), ct, base2);  // 1 - 1.5 usq + 4.5 ct^2
        const float2 a = __fmul2_rn(three, ct);
        const float2 ep = __fmul2_rn(w, __fadd2_rn(sym, a));
        const float2 en = __fmul2_rn(w, __fadd2_rn(sym, make_float2(-a.x, -a.y)));
        const float2 qp = rel2(__fadd2_rn(ep, make_float2(-v[i0], -v[i1])));
        const float2 qn = rel2(__fadd2_rn(en, make_float2(-v[j0], -v[j1])));
        v[i0] = __fadd_rn(v[i0], qp.x);
        v[i1] = __fadd_rn(v[i1], qp.y);
        v[j0] = __fadd_rn(v[j0], qn.x);
        v[j1] = __fadd_rn(v[j1], qn.y);
    });
    {
        constexpr int i = pair_rep(12), j = opp27(i);
        const float ct = cdot<i>(ux, uy, uz), w = wr[wclass(i)];
        const float sym = __fmaf_rn(__fmul_rn(4.5f, ct), ct, base), a = __fmul_rn(3.0f, ct);
        v[i] = __fadd_rn(v[i], rel(__fsub_rn(__fmul_rn(w, __fadd_rn(sym, a)), v[i])));
        v[j] = __fadd_rn(v[j], rel(__fsub_rn(__fmul_rn(w, __fsub_rn(sym, a)), v[j])));
    }
}

// equilibrium evaluations of the kernels' EQ template parameter (lbm_set_equilibrium_evaluation)
constexpr int EQ_FF = LBM_EQ_FLOAT_FLOAT, EQ_F64 = LBM_EQ_FP64, EQ_F32 = LBM_EQ_FP32;

struct StepArgs {
    const float *src;
    float *dst;
    const uint8_t *flags;
    Dims d;
    Tau tau;
    const float *induced;    // nullptr: no flow
    int cli;                 // 1: stream, reflect, collide, flow; 0: stream, collide
    const float *gathered;   // CLI order: the gather targets' populations (27 per target), or nullptr
    const int32_t *tgt_index;  // per cell: its row of `gathered`
};

// The fused kernel is launched as the gather kernel's programmatic dependent (pdl.cuh): it may launch
// as soon as every gather block has started and waits for the gather grid only in the threads that
// read a gathered row, so the other cells' blocks take the SMs the gather blocks leave and the
// launch gap between the two kernels disappears.

// one cell of the fused step: pull (or, for a target of the gather lists, its gathered populations),
// zero internal cells, collide, flow source, store
template <int EQ>
__device__ __forceinline__ bool fused_cell(const StepArgs &a, int64_t c, int x, int y, int z, uint8_t fl) {
    float v[27];
    if (a.cli && (fl & F_GATHER)) {
        // the row was written by this step's gather grid, which may still run: wait for it, then read
        // through L2 (not the read-only path: the row changed while this grid was resident)
        wait_prerequisite_grids();
        const float *g = a.gathered + (int64_t)__ldg(a.tgt_index + c) * 27;
#pragma unroll
        for (int j = 0; j < 27; ++j) v[j] = __ldcg(g + j);
    } else {
        pull(a.src, a.d, c, x, y, z, v);
    }
    if (a.cli && (fl & F_INTERNAL)) {
#pragma unroll
        for (int j = 0; j < 27; ++j) v[j] = 0.0f;
    }
    if constexpr (EQ == EQ_F32)
        collide_fp32(v, a.tau);
    else if (!collide<EQ == EQ_F64>(v, a.tau))
        return false;
    if (a.cli && a.induced && (fl & F_SOURCE)) {
#pragma unroll
        for (int j = 0; j < 27; ++j) v[j] = v[j] + __ldg(a.induced + j);
    }
#pragma unroll
    for (int j = 0; j < 27; ++j) a.dst[(int64_t)j * a.d.n + c] = v[j];
    return true;
}

// the rare cell whose float-float equilibrium the bound could not decide, recomputed in FP64
__device__ __noinline__ void fused_cell_fp64(StepArgs a, int64_t c, int x, int y, int z, uint8_t fl) {
    fused_cell<EQ_F64>(a, c, x, y, z, fl);
}

// 128-thread blocks, registers bounded for 5 per SM (20 warps): the paired float-float evaluation
// needs ~100 registers without spilling; the FP32 equilibrium fits 8 blocks per SM (32 warps)
constexpr int FUSED_THREADS = 128;
__host__ __device__ constexpr int fused_min_blocks(int eq) { return eq == EQ_F32 ? 8 : 5; }

// FP32-equilibrium step: the first thread of a block prefetches into L2 the 27 pulled segments of
// the block D3_PREFETCH_BLOCKS further on (`cp.async.bulk.prefetch.L2`, nothing held or awaited).
// A segment is rounded out to 16-byte boundaries of the population buffer (one allocation of 27
// planes) and clamped into it.  Measured on the 128^3 sphere model: 23.7k -> 24.3k MLUPS (32 to 256
// blocks ahead within 0.3 %); the float-float kernel measured slower with it (13.7k -> 10.9k), so it
// has none.
constexpr int D3_PREFETCH_BLOCKS = 128;

__device__ __forceinline__ void prefetch_block_ahead(const StepArgs &a) {
    if (threadIdx.x != 0) return;
    const int64_t first = ((int64_t)blockIdx.x + D3_PREFETCH_BLOCKS) * blockDim.x;
    const int64_t len = (int64_t)blockDim.x + 4;  // cells: the segment and a one-cell shift either way
    const int64_t total = 27 * a.d.n;             // elements of the buffer
    if (first + (int64_t)blockDim.x > a.d.n || total < len) return;
    Unroll<27>::run([&](auto jj) {
        constexpr int j = decltype(jj)::value;
        const int64_t off = (int64_t)kd(j, 2) + (int64_t)a.d.Z * ((int64_t)kd(j, 1) + (int64_t)a.d.Y * kd(j, 0));
        int64_t e = (int64_t)j * a.d.n + first - off;
        e = e < 0 ? 0 : (e > total - len ? total - len : e);
        e &= ~(int64_t)3;  // 16-byte aligned (the buffer itself is)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a.src + e), "r"((unsigned)(len * 4))
                     : "memory");
    });
}

template <int EQ>
__global__ void __launch_bounds__(FUSED_THREADS, fused_min_blocks(EQ)) fused_kernel(StepArgs a) {
    // one thread of the last block waits for the gather grid whatever the flags say, so this grid
    // never completes before it (work queued after the step sees the force the gather added)
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) wait_prerequisite_grids();
    allow_dependent_launch();  // the next step's gather kernel may launch (it waits for this grid)
    if constexpr (EQ == EQ_F32) prefetch_block_ahead(a);
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= a.d.n) return;
    const uint8_t fl = a.flags[c];
    int x, y, z;
    decode(a.d, c, x, y, z);
    if (!fused_cell<EQ>(a, c, x, y, z, fl)) fused_cell_fp64(a, c, x, y, z, fl);
}

struct GatherArgs {
    const int32_t *tgt;
    const int32_t *off;
    const GatherEntry *ent;
    int64_t ntgt;
    double *partials;  // 3 per block, or nullptr when no force is accumulated
    int force_mode;
    float *gathered;   // mode 0: the targets' populations out (27 per target)
    unsigned *done;    // blocks that have written their force partial (the last one finalises; 0 between launches)
    double *force;     // running force sum (3 doubles), the step's force added by the last block
    double *force_copy;  // if not null: the running sum after this launch also goes here
};

// force contribution m * (c_d SPLIT[d] - c_k SPLIT[k]) (SimCalcFuncs.cu:181-183); cs[j][a] = c_ja SPLIT_j
// (exact products), read from shared memory: the lanes of a warp index it with different directions,
// which the constant cache would serve one address at a time
__device__ __forceinline__ void force_term(float m, const GatherEntry &e, int mode, const float (*cs)[3],
                                           float acc[3]) {
    const int k = mode == LBM_FORCE_MOMENTUM_EXCHANGE ? e.slot / 3 : e.slot;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float kin = k < 27 ? cs[k][a] : 0.0f;
        const float coef = __fsub_rn(cs[e.dst_pop][a], kin);
        acc[a] = __fadd_rn(acc[a], __fmul_rn(m, coef));
    }
}

// The gather lists, one warp per target cell: lane j (< 27) holds population j of the cell -- pulled
// from its neighbour with zero fill (mode 0: the fused step, whose reflecting cells contribute their
// streamed populations) or read in place (mode 1: the reference's separate reflection pass) -- and
// the lanes read up to 32 of the cell's entries at once: each computes its contribution m = val * w
// and the warp walks them in list order, lane dst_pop adding each one that targets it, so every
// population takes its adds in the order of the sequential scatter (one rounded add of the rounded
// product per contribution, as the reference's atomicAdd at SimCalcFuncs.cu:177).  The force terms of
// a target are summed in FP32 by a fixed shuffle tree (the reference accumulates them with FP32
// atomics), the targets of a block in FP64 in warp order -- few FP64 instructions, which GB300 issues
// at a small fraction of its FP32 rate -- and the blocks by the FP64 finaliser.  Internal cells are
// zeroed.
// Mode 0 writes the result to the target's row of g.gathered, from which the fused kernel, launched
// next, collides the cell with all the others; mode 1 writes it to the destination lattice.
__device__ __forceinline__ float pull_one(const float *__restrict__ src, const Dims &d, int64_t c, int x, int y,
                                          int z, int j, const int (*dir)[3]) {
    const int sx = x - dir[j][0], sy = y - dir[j][1], sz = z - dir[j][2];
    if (sx < 0 || sy < 0 || sz < 0 || sx >= d.X || sy >= d.Y || sz >= d.Z) return 0.0f;
    return __ldg(src + (int64_t)j * d.n + sz + (int64_t)d.Z * (sy + (int64_t)d.Y * sx));
}

// sixteen target cells per block: fewer per-block force partials for the FP64 finaliser
constexpr int GATHER_THREADS = 512;

template <int MODE>
__global__ void __launch_bounds__(GATHER_THREADS) gather_kernel(StepArgs a, GatherArgs g) {
    // mode 0 is the programmatic dependent of the step before (its populations are read here) and
    // lets this step's fused kernel launch, which waits for the rows
    wait_prerequisite_grids();
    if (MODE == 0) allow_dependent_launch();
    // the direction tables in shared memory: each lane indexes them with its own direction
    __shared__ int s_dir[27][3];
    __shared__ float s_cs[27][3];
    if (threadIdx.x < 27) {
        for (int q = 0; q < 3; ++q) {
            s_dir[threadIdx.x][q] = c_dir[threadIdx.x][q];
            s_cs[threadIdx.x][q] = (float)c_dir[threadIdx.x][q] * c_split[threadIdx.x];
        }
    }
    __syncthreads();
    __shared__ double s_force[GATHER_THREADS / 32][3];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;  // target of this warp
    float facc[3] = {0.0f, 0.0f, 0.0f};
    if (i < g.ntgt) {  // uniform per warp
        const int64_t c = g.tgt[i];
        const uint8_t fl = a.flags[c];
        int x = 0, y = 0, z = 0;
        if (MODE == 0) decode(a.d, c, x, y, z);
        float v = 0.0f;  // population `lane` of the cell
        if (lane < 27)
            v = MODE == 0 ? pull_one(a.src, a.d, c, x, y, z, lane, s_dir) : __ldg(a.src + (int64_t)lane * a.d.n + c);
        const int k0 = g.off[i], k1 = g.off[i + 1];
        for (int base = k0; base < k1; base += 32) {
            const int k = base + lane;
            float m = 0.0f;
            int dst = 0;
            if (k < k1) {
                const GatherEntry e = g.ent[k];
                const int64_t s = MODE == 0 ? (int64_t)e.src_stream : (int64_t)e.src_cell;
                const float val = s >= 0 ? __ldg(a.src + (int64_t)e.src_pop * a.d.n + s) : 0.0f;
                m = __fmul_rn(val, e.w);
                dst = e.dst_pop;
                if (g.partials) force_term(m, e, g.force_mode, s_cs, facc);
            }
            const int cnt = min(32, k1 - base);
            for (int j = 0; j < cnt; ++j) {
                const float mj = __shfl_sync(0xffffffffu, m, j);
                const int dj = __shfl_sync(0xffffffffu, dst, j);
                if (lane == dj) v = __fadd_rn(v, mj);
            }
        }
        if (fl & F_INTERNAL) v = 0.0f;
        if (lane < 27) {
            if (MODE == 0)
                g.gathered[i * 27 + lane] = v;
            else
                a.dst[(int64_t)lane * a.d.n + c] = v;
        }
    }
    if (g.partials) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) facc[q] = __fadd_rn(facc[q], __shfl_xor_sync(0xffffffffu, facc[q], o));
            if (lane == 0) s_force[warp][q] = (double)facc[q];
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            double t = 0.0;
            for (int w = 0; w < GATHER_THREADS / 32; ++w) t += s_force[w][threadIdx.x];
            g.partials[3 * blockIdx.x + threadIdx.x] = t;
            __threadfence();  // the partial is visible device-wide before this block is counted
        }
        // the last block to finish adds the partials of all blocks, in a fixed order whichever block
        // that is: thread t the blocks t, t + GATHER_THREADS, ..., then a tree over the threads
        __shared__ bool s_last;
        __shared__ double s_sum[3][GATHER_THREADS];
        __syncthreads();
        if (threadIdx.x == 0) s_last = atomicAdd(g.done, 1u) == gridDim.x - 1;
        __syncthreads();
        if (s_last) {
            __threadfence();
            for (int q = 0; q < 3; ++q) {
                double t = 0.0;
                for (unsigned b = threadIdx.x; b < gridDim.x; b += GATHER_THREADS) t += __ldcg(g.partials + 3 * b + q);
                s_sum[q][threadIdx.x] = t;
            }
            __syncthreads();
            for (int h = GATHER_THREADS / 2; h > 0; h >>= 1) {
                if ((int)threadIdx.x < h)
                    for (int q = 0; q < 3; ++q) s_sum[q][threadIdx.x] += s_sum[q][threadIdx.x + h];
                __syncthreads();
            }
            if (threadIdx.x < 3) {
                const double v = g.force[threadIdx.x] + s_sum[threadIdx.x][0];
                g.force[threadIdx.x] = v;
                if (g.force_copy) g.force_copy[threadIdx.x] = v;
            }
            if (threadIdx.x == 0) *g.done = 0;  // ready for the next launch (stream-ordered)
        }
    }
}

// ------------------------------------------------------------------------- separate passes
__global__ void stream_kernel(const float *__restrict__ src, float *__restrict__ dst, Dims d) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    int x, y, z;
    decode(d, c, x, y, z);
    float v[27];
    pull(src, d, c, x, y, z, v);
#pragma unroll
    for (int j = 0; j < 27; ++j) dst[(int64_t)j * d.n + c] = v[j];
}

// reflection pass for cells that receive nothing: copy, internal cells zeroed
__global__ void reflect_copy_kernel(const float *__restrict__ src, float *__restrict__ dst,
                                    const uint8_t *__restrict__ flags, Dims d) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const uint8_t fl = flags[c];
    if (fl & F_GATHER) return;
    const bool zero = fl & F_INTERNAL;
#pragma unroll
    for (int j = 0; j < 27; ++j) dst[(int64_t)j * d.n + c] = zero ? 0.0f : __ldg(src + (int64_t)j * d.n + c);
}

template <int EQ>
__global__ void collide_kernel(float *__restrict__ f, Dims d, Tau tau) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    float v[27];
#pragma unroll
    for (int j = 0; j < 27; ++j) v[j] = f[(int64_t)j * d.n + c];
    if constexpr (EQ == EQ_F32) {
        collide_fp32(v, tau);
    } else if (!collide<EQ == EQ_F64>(v, tau)) {  // undecided by the float-float bound: the cell again in FP64
#pragma unroll
        for (int j = 0; j < 27; ++j) v[j] = f[(int64_t)j * d.n + c];
        collide<true>(v, tau);
    }
#pragma unroll
    for (int j = 0; j < 27; ++j) f[(int64_t)j * d.n + c] = v[j];
}

__global__ void flow_kernel(float *__restrict__ f, const uint8_t *__restrict__ flags, Dims d,
                            const float *__restrict__ induced) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= d.n || !(flags[c] & F_SOURCE)) return;
#pragma unroll
    for (int j = 0; j < 27; ++j) f[(int64_t)j * d.n + c] = f[(int64_t)j * d.n + c] + induced[j];
}

// ------------------------------------------------------------------------- results and I/O
__global__ void moments_kernel(const float *__restrict__ f, Dims d, float *rho, float *ux, float *uy, float *uz) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    float density = 0.0f, vx = 0.0f, vy = 0.0f, vz = 0.0f;
    Unroll<27>::run([&](auto ii) {
        constexpr int i = decltype(ii)::value;
        const float v = f[(int64_t)i * d.n + c];
        density += v;
        split_moment<i>(v, vx, vy, vz);
    });
    if (density != 0.0f) {
        vx /= density;
        vy /= density;
        vz /= density;
    }
    if (rho) rho[c] = density;
    if (ux) ux[c] = vx;
    if (uy) uy[c] = vy;
    if (uz) uz[c] = vz;
}

__global__ void conservation_kernel(const float *__restrict__ f, const uint8_t *__restrict__ flags, Dims d,
                                    double *partials) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < d.n; c += (int64_t)gridDim.x * blockDim.x) {
        if (flags[c] & F_INTERNAL) continue;
#pragma unroll
        for (int i = 0; i < 27; ++i) {
            const double v = f[(int64_t)i * d.n + c];
            acc[0] += v;
            acc[1] += v * c_dir[i][0];
            acc[2] += v * c_dir[i][1];
            acc[3] += v * c_dir[i][2];
        }
    }
    block_sum<4>(acc, partials + 4 * blockIdx.x);
}

// host layouts: cell-major [cell][27] float/double, or LatticePoint records (144 bytes; floats
// from byte 12, flags at 120 / 121, pointers at 128 / 136)
template <class H>
__global__ void load_kernel(float *__restrict__ f, const H *__restrict__ host, Dims d, int aos) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    for (int j = 0; j < 27; ++j) {
        float v;
        if (aos)
            v = reinterpret_cast<const float *>(reinterpret_cast<const char *>(host) + c * 144 + 12)[j];
        else
            v = (float)host[c * 27 + j];
        f[(int64_t)j * d.n + c] = v;
    }
}

template <class H>
__global__ void store_kernel(const float *__restrict__ f, H *__restrict__ host, const uint8_t *__restrict__ flags,
                             Dims d, int aos) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    if (aos) {
        char *rec = reinterpret_cast<char *>(host) + c * 144;
        int x, y, z;
        decode(d, c, x, y, z);
        int *xyz = reinterpret_cast<int *>(rec);
        xyz[0] = x;
        xyz[1] = y;
        xyz[2] = z;
        float *p = reinterpret_cast<float *>(rec + 12);
        for (int j = 0; j < 27; ++j) p[j] = f[(int64_t)j * d.n + c];
        const uint8_t fl = flags[c];
        rec[120] = (fl & LBM_REFLECTED) ? 1 : 0;
        rec[121] = (fl & LBM_INTERNAL) ? 1 : 0;
        rec[122] = rec[123] = 0;
        *reinterpret_cast<int *>(rec + 124) = 0;
        *reinterpret_cast<unsigned long long *>(rec + 128) = 0ull;
        *reinterpret_cast<unsigned long long *>(rec + 136) = 0ull;
    } else {
        for (int j = 0; j < 27; ++j) host[c * 27 + j] = (H)f[(int64_t)j * d.n + c];
    }
}

inline Dims dims(const lbm_ctx *ctx) {
    return Dims{ctx->desc.nx, ctx->desc.ny, ctx->desc.nz, ctx->cells, FastDiv::make((uint32_t)ctx->desc.nz),
                FastDiv::make((uint32_t)ctx->desc.ny)};
}

inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

float *cur(lbm_ctx *ctx) { return static_cast<float *>(ctx->f[ctx->cur]); }
float *nxt(lbm_ctx *ctx) { return static_cast<float *>(ctx->f[ctx->cur ^ 1]); }

// Tau of the context, with RN(1/tau) and the outcome of the exhaustive division check, cached per
// tau value for the process (the check runs once per value, a few milliseconds on the GPU).
Tau tau_of(lbm_ctx *ctx) {
    static std::mutex mu;
    static std::map<uint32_t, std::pair<float, int>> cache;
    const float b = ctx->desc.tau;
    uint32_t key;
    std::memcpy(&key, &b, sizeof(key));
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = cache.find(key);
        if (it != cache.end()) return Tau{b, it->second.first, it->second.second};
    }
    Tau t{b, 0.0f, 0};
    const float ab = std::fabs(b);
    if (!(ab >= 0x1p-60f && ab <= 0x1p60f)) return t;  // keep the IEEE division for extreme tau
    void *buf = nullptr;
    if (cudaMalloc(&buf, 16) != cudaSuccess) {
        cudaGetLastError();
        return t;
    }
    float *y_d = static_cast<float *>(buf);
    unsigned long long *bad_d = reinterpret_cast<unsigned long long *>(static_cast<char *>(buf) + 8);
    float y = 0.0f;
    unsigned long long bad = 1;
    cudaError_t e = cudaMemsetAsync(buf, 0, 16, ctx->stream);
    if (e == cudaSuccess) {
        tau_check_kernel<<<1216, 256, 0, ctx->stream>>>(b, y_d, bad_d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&y, y_d, sizeof(y), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, bad_d, sizeof(bad), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(buf);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return t;
    }
    t.y = y;
    t.fast = bad == 0 ? 1 : 0;
    std::lock_guard<std::mutex> g(mu);
    cache[key] = {t.y, t.fast};
    return t;
}

GatherArgs gather_args(lbm_ctx *ctx) {
    GatherArgs g;
    g.tgt = ctx->tgt_cells_d;
    g.off = ctx->tgt_off_d;
    g.ent = ctx->entries_d;
    g.ntgt = ctx->ntgt;
    g.partials = ctx->force_on ? ctx->scratch.partials : nullptr;
    g.force_mode = ctx->desc.force_mode;
    g.gathered = ctx->gathered_d;
    g.done = ctx->gather_done_d;
    g.force = ctx->force_acc_d;
    g.force_copy = nullptr;
    return g;
}

cudaError_t launch_gather(lbm_ctx *ctx, const StepArgs &a, int mode, double *force_copy = nullptr) {
    if (ctx->ntgt == 0) return cudaSuccess;
    GatherArgs g = gather_args(ctx);
    g.force_copy = force_copy;
    const int threads = GATHER_THREADS;
    const unsigned nb = (unsigned)d3q27_gather_blocks(ctx->ntgt);  // one warp per target cell
    static_assert(GATHER_THREADS == 16 * 32, "d3q27_gather_blocks assumes sixteen warps per block");
    if (mode != 0) {
        gather_kernel<1><<<nb, threads, 0, ctx->stream>>>(a, g);
        return cudaGetLastError();
    }
    // the step's gather: the programmatic dependent of the launch before (the previous step's fused
    // kernel), its blocks waiting for that grid at entry
    const cudaError_t e = launch_maybe_dependent(true, gather_kernel<0>, dim3(nb), dim3(threads), 0, ctx->stream, a, g);
    return e != cudaSuccess ? e : cudaGetLastError();  // the force, when accumulated, was added by the kernel's last block
}

// Both equilibrium evaluations on n pseudo-random (rho, u) samples, all directions: counts the
// float-float results accepted by their bound that differ from FP64 (out[0]; the single evaluator
// and both signs of the pair evaluator), and the pair evaluations left to the FP64 fallback among
// samples with |u| <= 0.05 (out[1]).
__global__ void eq_selftest_kernel(int64_t n, uint64_t seed, unsigned long long *out) {
    unsigned long long bad = 0, fell = 0;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        // SplitMix64 stream per sample; magnitudes spread over decades, velocities up to |u| ~ 2
        uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(s + 1);
        float r[5];
        for (int k = 0; k < 5; ++k) {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t t = z;
            t = (t ^ (t >> 30)) * 0xBF58476D1CE4E5B9ull;
            t = (t ^ (t >> 27)) * 0x94D049BB133111EBull;
            t ^= t >> 31;
            r[k] = (float)(t >> 40) * 0x1p-24f;  // [0, 1)
        }
        const float scale = exp2f(floorf(r[4] * 16.0f) - 8.0f);
        const float rho = (0.01f + 2.0f * r[0]) * scale;
        const float umax = (s & 3) == 0 ? 2.0f : ((s & 3) == 1 ? 0.3f : ((s & 3) == 2 ? 0.05f : 1e-3f));
        const float ux = (2.0f * r[1] - 1.0f) * umax, uy = (2.0f * r[2] - 1.0f) * umax;
        const float uz = (2.0f * r[3] - 1.0f) * umax * ((s & 4) ? 1.0f : 0.0f);
        const float usq = (ux * ux) + (uy * uy) + (uz * uz);
        const float c1 = __fmul_rn(1.5f, usq), c1e = __fmaf_rn(1.5f, usq, -c1);
        // the pair evaluator of the step, both signs
        for (int i = 1; i < 27; ++i) {
            const int k = wclass(i);
            const float ph = __fmul_rn(kWhi(k), rho);
            const float pl = __fmaf_rn(kWlo(k), rho, __fmaf_rn(kWhi(k), rho, -ph));
            const float ct = __fadd_rn(__fadd_rn((float)c_dir[i][0] * ux, (float)c_dir[i][1] * uy), (float)c_dir[i][2] * uz);
            float rp, rn;
            bool okp, okn;
            eq_ff_pair(ph, pl, __fmul_rn(fabsf(ph), 0x1p-42f), c1, c1e, __fadd_rn(1.0f, c1), ct, rp, okp, rn, okn);
            bad += okp && __float_as_uint(rp) != __float_as_uint(eq_fp64(k, rho, ct, usq));
            bad += okn && __float_as_uint(rn) != __float_as_uint(eq_fp64(k, rho, -ct, usq));
            fell += !okp && (s & 3) >= 2;  // fallbacks counted for |u| <= 0.05 (low-Mach flows)
            // the paired form, lane x this direction and lane y the next one: the same bits and
            // flags as the scalar evaluation of each
            const int i2 = i % 26 + 1, k2 = wclass(i2);
            const float ph2 = __fmul_rn(kWhi(k2), rho);
            const float pl2 = __fmaf_rn(kWlo(k2), rho, __fmaf_rn(kWhi(k2), rho, -ph2));
            const float ct2 = __fadd_rn(__fadd_rn((float)c_dir[i2][0] * ux, (float)c_dir[i2][1] * uy), (float)c_dir[i2][2] * uz);
            float rp2, rn2;
            bool okp2, okn2;
            eq_ff_pair(ph2, pl2, __fmul_rn(fabsf(ph2), 0x1p-42f), c1, c1e, __fadd_rn(1.0f, c1), ct2, rp2, okp2, rn2, okn2);
            float2 vp, vn;
            Ok2 op, on;
            eq_ff_pair(make_float2(ph, ph2), make_float2(pl, pl2),
                       make_float2(__fmul_rn(fabsf(ph), 0x1p-42f), __fmul_rn(fabsf(ph2), 0x1p-42f)), make_float2(c1, c1),
                       make_float2(c1e, c1e), make_float2(__fadd_rn(1.0f, c1), __fadd_rn(1.0f, c1)), make_float2(ct, ct2),
                       vp, op, vn, on);
            bad += __float_as_uint(vp.x) != __float_as_uint(rp) || __float_as_uint(vn.x) != __float_as_uint(rn) ||
                   op.x != okp || on.x != okn;
            bad += __float_as_uint(vp.y) != __float_as_uint(rp2) || __float_as_uint(vn.y) != __float_as_uint(rn2) ||
                   op.y != okp2 || on.y != okn2;
        }
        for (int i = 0; i < 27; ++i) {
            const int k = wclass(i);
            const float ph = __fmul_rn(kWhi(k), rho);
            const float pl = __fmaf_rn(kWlo(k), rho, __fmaf_rn(kWhi(k), rho, -ph));
            const float ct = __fadd_rn(__fadd_rn((float)c_dir[i][0] * ux, (float)c_dir[i][1] * uy), (float)c_dir[i][2] * uz);
            bool ok;  // (c_i . u with the table in constant memory: the same value as cdot<i>)
            const float a = eq_ff(ph, pl, c1, c1e, ct, ok);
            const float b = eq_fp64(k, rho, ct, usq);
            bad += ok && __float_as_uint(a) != __float_as_uint(b);
        }
    }
    atomicAdd(out, bad);
    atomicAdd(out + 1, fell);
}

}  // namespace

cudaError_t d3q27_division_check(float tau, unsigned long long *bad_d, float *y_d, cudaStream_t st) {
    tau_check_kernel<<<1216, 256, 0, st>>>(tau, y_d, bad_d);
    return cudaGetLastError();
}

cudaError_t d3q27_eq_selftest(int64_t n, uint64_t seed, unsigned long long *out_d, cudaStream_t st) {
    eq_selftest_kernel<<<1216, 256, 0, st>>>(n, seed, out_d);
    return cudaGetLastError();
}

cudaError_t d3q27_step(lbm_ctx *ctx, int nsteps, double *series_d) {
    const int threads = FUSED_THREADS;
    const Tau tau = tau_of(ctx);
    const Dims dm = dims(ctx);
    for (int s = 0; s < nsteps; ++s) {
        StepArgs a;
        a.src = cur(ctx);
        a.dst = nxt(ctx);
        a.flags = ctx->flags_d;
        a.d = dm;
        a.tau = tau;
        a.cli = ctx->desc.order == LBM_ORDER_CLI;
        a.induced = (a.cli && ctx->flow_on) ? ctx->induced_d : nullptr;
        a.gathered = ctx->gathered_d;
        a.tgt_index = ctx->tgt_index_d;
        cudaError_t e = cudaSuccess;
        double *copy = series_d ? series_d + 3 * (int64_t)s : nullptr;
        const bool reduced = a.cli && ctx->ntgt > 0 && ctx->force_on;  // the force changes this step
        const bool gathered = a.cli && ctx->ntgt > 0;
        if (a.cli) {  // the targets of the gather lists first: the fused kernel collides them
            e = launch_gather(ctx, a, 0, copy);
            if (e != cudaSuccess) return e;
        }
        // after a gather launch the fused kernel is its programmatic dependent (it overlaps the
        // gather's tail); otherwise an ordinary stream-ordered launch
        const dim3 grid(blocks_for(ctx->cells, threads)), block(threads);
        if (ctx->eq_mode == EQ_F64)
            e = launch_maybe_dependent(gathered, fused_kernel<EQ_F64>, grid, block, 0, ctx->stream, a);
        else if (ctx->eq_mode == EQ_F32)
            e = launch_maybe_dependent(gathered, fused_kernel<EQ_F32>, grid, block, 0, ctx->stream, a);
        else
            e = launch_maybe_dependent(gathered, fused_kernel<EQ_FF>, grid, block, 0, ctx->stream, a);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (copy && !reduced) {
            e = cudaMemcpyAsync(copy, ctx->force_acc_d, 3 * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream);
            if (e != cudaSuccess) return e;
        }
        ctx->cur ^= 1;
    }
    return cudaSuccess;
}

cudaError_t d3q27_apply(lbm_ctx *ctx, int op) {
    const int threads = 256;
    const Dims d = dims(ctx);
    const unsigned nb = blocks_for(ctx->cells, threads);
    cudaError_t e = cudaSuccess;
    switch (op) {
        case LBM_OP_STREAM:
            stream_kernel<<<nb, threads, 0, ctx->stream>>>(cur(ctx), nxt(ctx), d);
            e = cudaGetLastError();
            ctx->cur ^= 1;
            break;
        case LBM_OP_REFLECT: {
            reflect_copy_kernel<<<nb, threads, 0, ctx->stream>>>(cur(ctx), nxt(ctx), ctx->flags_d, d);
            e = cudaGetLastError();
            if (e != cudaSuccess) return e;
            StepArgs a;
            a.src = cur(ctx);
            a.dst = nxt(ctx);
            a.flags = ctx->flags_d;
            a.d = d;
            a.tau = tau_of(ctx);
            a.induced = nullptr;
            a.cli = 1;
            a.gathered = nullptr;
            a.tgt_index = nullptr;
            e = launch_gather(ctx, a, 1);
            ctx->cur ^= 1;
            break;
        }
        case LBM_OP_COLLIDE:
            if (ctx->eq_mode == EQ_F64)
                collide_kernel<EQ_F64><<<nb, threads, 0, ctx->stream>>>(cur(ctx), d, tau_of(ctx));
            else if (ctx->eq_mode == EQ_F32)
                collide_kernel<EQ_F32><<<nb, threads, 0, ctx->stream>>>(cur(ctx), d, tau_of(ctx));
            else
                collide_kernel<EQ_FF><<<nb, threads, 0, ctx->stream>>>(cur(ctx), d, tau_of(ctx));
            e = cudaGetLastError();
            break;
        case LBM_OP_FLOW:
            if (ctx->flow_on) {
                flow_kernel<<<nb, threads, 0, ctx->stream>>>(cur(ctx), ctx->flags_d, d, ctx->induced_d);
                e = cudaGetLastError();
            }
            break;
        default:
            return cudaErrorInvalidValue;
    }
    return e;
}

cudaError_t d3q27_moments(lbm_ctx *ctx, float *rho_d, float *ux_d, float *uy_d, float *uz_d) {
    moments_kernel<<<blocks_for(ctx->cells, 256), 256, 0, ctx->stream>>>(cur(ctx), dims(ctx), rho_d, ux_d, uy_d, uz_d);
    return cudaGetLastError();
}

cudaError_t d3q27_conservation(lbm_ctx *ctx, double *out_d) {
    const int nblocks = 512;
    conservation_kernel<<<nblocks, 256, 0, ctx->stream>>>(cur(ctx), ctx->flags_d, dims(ctx), ctx->scratch.partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return finalize_sums(ctx->stream, ctx->scratch.partials, nblocks, 4, out_d);
}

cudaError_t d3q27_load(lbm_ctx *ctx, const void *src_d, int src_dtype, int aos) {
    const unsigned nb = blocks_for(ctx->cells, 128);
    if (aos || src_dtype == LBM_F32)
        load_kernel<float><<<nb, 128, 0, ctx->stream>>>(cur(ctx), static_cast<const float *>(src_d), dims(ctx), aos);
    else
        load_kernel<double><<<nb, 128, 0, ctx->stream>>>(cur(ctx), static_cast<const double *>(src_d), dims(ctx), 0);
    return cudaGetLastError();
}

cudaError_t d3q27_store(lbm_ctx *ctx, void *dst_d, int dst_dtype, int aos) {
    const unsigned nb = blocks_for(ctx->cells, 128);
    if (aos || dst_dtype == LBM_F32)
        store_kernel<float><<<nb, 128, 0, ctx->stream>>>(cur(ctx), static_cast<float *>(dst_d), ctx->flags_d, dims(ctx), aos);
    else
        store_kernel<double><<<nb, 128, 0, ctx->stream>>>(cur(ctx), static_cast<double *>(dst_d), ctx->flags_d, dims(ctx), 0);
    return cudaGetLastError();
}

}  // namespace lbm
