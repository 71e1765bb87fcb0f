/*
 * lbm_oracle.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU restatement of the lattice Boltzmann step that the GPU library implements. It is the
 * checker for the parity tests (tests/), for __graft_entry__.smoke() and for the cpu_baseline
 * leg of bench.py, and nothing else: the product library never links, loads or calls it.
 *
 * Two halves:
 *
 *  1. D3Q27 "reference" step.  A literal restatement of the reference kernels in
 *     simulation/source/SimCalcFuncs.cu, one function per kernel, on cell-major arrays
 *     f[cell * 27 + q] with the reference host cell index  z + Z*(y + Y*x)
 *     (simulation/source/Lattice.cpp:254,340,447):
 *        orc_d3q27_stream   <- CudaFunctions::calculate_streaming   SimCalcFuncs.cu:79-96
 *        orc_d3q27_collide  <- CudaFunctions::calculate_collision   SimCalcFuncs.cu:98-156
 *        orc_d3q27_reflect  <- CudaFunctions::calculate_reflections SimCalcFuncs.cu:158-198
 *        orc_d3q27_flow     <- CudaFunctions::generate_flow         SimCalcFuncs.cu:200-215
 *     and the step orders of Lattice::simulateLattice (Lattice.cpp:222-226: stream, collide) and
 *     of the CLI loop (LatticeBoltzmannCuda.cpp:85-93: stream, reflect, collide, flow).
 *     Pinned against the known answers of test/CalculationsTest.cpp (see tests/golden/).
 *
 *  2. D2Q9 BGK step in FP64 and FP32: pull streaming of post-collision populations, half-way
 *     bounce-back at solid cells and non-periodic domain edges, moving-wall bounce-back, periodic
 *     wrap, Guo body force.  The reference has no D2Q9 code; this half is pinned by analytic
 *     solutions (Taylor-Green decay, Poiseuille profile) and by conservation, in tests/.
 *
 * Plain C11 + OpenMP; builds with gcc on x86_64 and aarch64 (no intrinsics).
 * Compile with -ffp-contract=off so that every product/sum is rounded separately.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------------ */
/* D3Q27 reference tables.  Same values and order as SimCalcFuncs.cu:12-14 (device copies) and  */
/* Constants.cpp:6-7 (host copies): rest, 6 faces, 12 edges, 8 corners.                        */
/* ------------------------------------------------------------------------------------------ */
static const int C27[27][3] = {
    {0, 0, 0},   {-1, 0, 0},  {0, -1, 0},  {0, 0, -1},  {0, 0, 1},    {0, 1, 0},    {1, 0, 0},
    {-1, -1, 0}, {-1, 0, -1}, {-1, 0, 1},  {-1, 1, 0},  {0, -1, -1},  {0, -1, 1},   {0, 1, -1},
    {0, 1, 1},   {1, -1, 0},  {1, 0, -1},  {1, 0, 1},   {1, 1, 0},    {-1, -1, -1}, {-1, -1, 1},
    {-1, 1, -1}, {-1, 1, 1},  {1, -1, -1}, {1, -1, 1},  {1, 1, -1},   {1, 1, 1}};
static const int INV27[27] = {0,  6,  5,  4,  3,  2,  1,  18, 17, 16, 15, 14, 13, 12,
                              11, 10, 9,  8,  7,  26, 25, 24, 23, 22, 21, 20, 19};
static const float SPLIT27[27] = {0.0f,        1.0f,        1.0f,        1.0f,        1.0f,
                                  1.0f,        1.0f,        0.5f,        0.5f,        0.5f,
                                  0.5f,        0.5f,        0.5f,        0.5f,        0.5f,
                                  0.5f,        0.5f,        0.5f,        0.5f,        1.0f / 3.0f,
                                  1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 3.0f,
                                  1.0f / 3.0f, 1.0f / 3.0f};

/* Per-cell reflection record, same layout as ReflectionValues (LatticePoint.h:3-7):
 * 81 slots, slot s = 3*population + k, direction packed 5 bits per slot, 6 slots per int. */
typedef struct {
    int32_t dirs[14];
    float w[81];
} orc_refl_values;

/* cell flag bits shared with the GPU library's D3Q27 mode */
enum { ORC_INTERNAL = 1, ORC_REFLECTED = 2, ORC_SOURCE = 4 };

static inline long cell27(int x, int y, int z, int Y, int Z) { return (long)z + (long)Z * ((long)y + (long)Y * x); }

/* 5-bit direction of slot s (Lattice.cpp:465-477, SimCalcFuncs.cu:18-30) */
int orc_refl_get_dir(const orc_refl_values *r, int s) {
    unsigned int word = (unsigned int)r->dirs[s / 6];
    return (int)((word >> (5 * (s % 6))) & 31u);
}

/* Lattice.cpp:450-463 */
void orc_refl_set_dir(orc_refl_values *r, int s, int dir) {
    unsigned int word = (unsigned int)r->dirs[s / 6];
    unsigned int sh = 5u * (unsigned int)(s % 6);
    word = (word & ~(31u << sh)) | (((unsigned int)dir & 31u) << sh);
    r->dirs[s / 6] = (int32_t)word;
}

/* Utils.cpp:4-29 (used only by the reference's CompressionTest) */
unsigned int orc_compress_ints(const int *a, int num, int bit_length) {
    unsigned int out = 0, max = 1;
    for (int b = 0; b < bit_length; ++b) max *= 2u;
    for (int i = 0; i < num - 1; ++i) {
        if ((unsigned int)a[i] < max) {
            out |= (unsigned int)a[i];
            out <<= 5;
        }
    }
    if ((unsigned int)a[num - 1] < max) out |= (unsigned int)a[num - 1];
    return out;
}

/* calculate_streaming, SimCalcFuncs.cu:79-96: pull from x + c_i into slot INV[i]; outside -> 0.
 * Equivalently dst[x][j] = src[x - c_j][j]. */
int orc_d3q27_stream(int X, int Y, int Z, const float *src, float *dst) {
#pragma omp parallel for schedule(static)
    for (int x = 0; x < X; ++x)
        for (int y = 0; y < Y; ++y)
            for (int z = 0; z < Z; ++z) {
                long c = cell27(x, y, z, Y, Z);
                for (int i = 0; i < 27; ++i) {
                    int nx = x + C27[i][0], ny = y + C27[i][1], nz = z + C27[i][2];
                    int j = INV27[i];
                    if (nx < 0 || ny < 0 || nz < 0 || nx >= X || ny >= Y || nz >= Z)
                        dst[c * 27 + j] = 0.0f;
                    else
                        dst[c * 27 + j] = src[cell27(nx, ny, nz, Y, Z) * 27 + j];
                }
            }
    return 0;
}

/* One cell of calculate_collision, SimCalcFuncs.cu:98-156.  Density and the SPLIT-weighted
 * velocity in FP32; equilibrium evaluated in FP64 (double literals) and rounded to float; the
 * BGK update f += (eq - f)/tau in FP32. */
static void d3q27_collide_cell(float *f, float tau) {
    float density = 0.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f;
    for (int i = 0; i < 27; ++i) {
        density += f[i];
        ux += f[i] * (float)C27[i][0] * SPLIT27[i];
        uy += f[i] * (float)C27[i][1] * SPLIT27[i];
        uz += f[i] * (float)C27[i][2] * SPLIT27[i];
    }
    if (density != 0.0f) {
        ux /= density;
        uy /= density;
        uz /= density;
    }
    float usq = (ux * ux) + (uy * uy) + (uz * uz);
    for (int i = 0; i < 27; ++i) {
        double wgt = i == 0 ? (8.0 / 27.0) : i < 7 ? (2.0 / 27.0) : i < 19 ? (1.0 / 54.0) : (1.0 / 216.0);
        float ct = ((float)C27[i][0] * ux) + ((float)C27[i][1] * uy) + ((float)C27[i][2] * uz);
        float eq = (float)(wgt * density * (1 + (3.0 * ct) + (4.5 * ct * ct) - (1.5 * usq)));
        float delta = (eq - f[i]) / tau;
        f[i] = f[i] + delta;
    }
}

int orc_d3q27_collide(int X, int Y, int Z, float *f, float tau) {
    long n = (long)X * Y * Z;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < n; ++c) d3q27_collide_cell(f + c * 27, tau);
    return 0;
}

/* calculate_reflections, SimCalcFuncs.cu:158-198.  dst starts as a copy of src (the temporary
 * lattice of Lattice.cpp:163-210).  Every reflected cell scatters f[s/3]*w[s] of slots 1..80 into
 * population dir(s) of its neighbour x + c_dir(s) in dst; internal cells are then zeroed in dst.
 * The optional force (SimCalcFuncs.cu:179-184) is m*(c_d*SPLIT[d] - c_k*SPLIT[k]):
 *   force_mode 0 (reference): k = s, the slot index, as the reference indexes DIRECTIONS[i] and
 *                SPLIT[i] with the slot; for s >= 27 the reference reads past its 27-entry tables
 *                (undefined), and this restatement takes that term as zero.
 *   force_mode 1 (momentum exchange): k = s/3, the population that arrived.
 * Cells are visited in x, y, z, slot order; the reference's float atomics have no fixed order. */
int orc_d3q27_reflect(int X, int Y, int Z, const float *src, float *dst, const uint8_t *flags,
                      const int32_t *tab_idx, const orc_refl_values *tabs, float *force,
                      int force_mode) {
    long n = (long)X * Y * Z;
    memcpy(dst, src, sizeof(float) * 27 * (size_t)n);
    for (int x = 0; x < X; ++x)
        for (int y = 0; y < Y; ++y)
            for (int z = 0; z < Z; ++z) {
                long c = cell27(x, y, z, Y, Z);
                if (!(flags[c] & ORC_REFLECTED) || tab_idx[c] < 0) continue;
                const orc_refl_values *r = &tabs[tab_idx[c]];
                for (int s = 1; s < 81; ++s) {
                    int d = orc_refl_get_dir(r, s);
                    if (d == 0) continue;
                    if (d > 26) return -1;
                    int nx = x + C27[d][0], ny = y + C27[d][1], nz = z + C27[d][2];
                    if (nx < 0 || ny < 0 || nz < 0 || nx >= X || ny >= Y || nz >= Z) continue;
                    float m = src[c * 27 + s / 3] * r->w[s];
                    long t = cell27(nx, ny, nz, Y, Z);
                    dst[t * 27 + d] += m;
                    if (force) {
                        int k = force_mode == 1 ? s / 3 : s;
                        float kx = 0.0f, ky = 0.0f, kz = 0.0f;
                        if (k < 27) {
                            kx = (float)C27[k][0] * SPLIT27[k];
                            ky = (float)C27[k][1] * SPLIT27[k];
                            kz = (float)C27[k][2] * SPLIT27[k];
                        }
                        force[0] += m * (((float)C27[d][0] * SPLIT27[d]) - kx);
                        force[1] += m * (((float)C27[d][1] * SPLIT27[d]) - ky);
                        force[2] += m * (((float)C27[d][2] * SPLIT27[d]) - kz);
                    }
                }
            }
    for (long c = 0; c < n; ++c)
        if (flags[c] & ORC_INTERNAL)
            for (int q = 0; q < 27; ++q) dst[c * 27 + q] = 0.0f;
    return 0;
}

/* generate_flow, SimCalcFuncs.cu:200-215: add the induced populations where the criterion
 * holds.  The criterion is given as the ORC_SOURCE flag bit, evaluated by the caller. */
int orc_d3q27_flow(int X, int Y, int Z, float *f, const uint8_t *flags, const float *induced) {
    long n = (long)X * Y * Z;
    for (long c = 0; c < n; ++c)
        if (flags[c] & ORC_SOURCE)
            for (int q = 0; q < 27; ++q) f[c * 27 + q] = f[c * 27 + q] + induced[q];
    return 0;
}

/* order 0: Lattice::simulateLattice (stream, collide), Lattice.cpp:222-226.
 * order 1: CLI loop (stream, reflect, collide, flow), LatticeBoltzmannCuda.cpp:85-93; reflect is
 *          skipped when tab_idx is NULL and flow when induced is NULL (the reference's
 *          m_flowData == nullptr check, Lattice.cpp:216). */
int orc_d3q27_run(int X, int Y, int Z, float *f, const uint8_t *flags, const int32_t *tab_idx,
                  const orc_refl_values *tabs, float tau, const float *induced, int order, int nsteps,
                  float *force, int force_mode) {
    long n = (long)X * Y * Z;
    float *tmp = (float *)malloc(sizeof(float) * 27 * (size_t)n);
    if (!tmp) return -3;
    int rc = 0;
    for (int s = 0; s < nsteps && rc == 0; ++s) {
        orc_d3q27_stream(X, Y, Z, f, tmp);
        memcpy(f, tmp, sizeof(float) * 27 * (size_t)n);
        if (order == 1 && tab_idx) {
            rc = orc_d3q27_reflect(X, Y, Z, f, tmp, flags, tab_idx, tabs, force, force_mode);
            memcpy(f, tmp, sizeof(float) * 27 * (size_t)n);
        }
        orc_d3q27_collide(X, Y, Z, f, tau);
        if (order == 1 && induced) orc_d3q27_flow(X, Y, Z, f, flags, induced);
    }
    free(tmp);
    return rc;
}

/* ------------------------------------------------------------------------------------------ */
/* D2Q9.  Population order (shared with the GPU library):                                     */
/*   0:(0,0) 1:(1,0) 2:(0,1) 3:(-1,0) 4:(0,-1) 5:(1,1) 6:(-1,1) 7:(-1,-1) 8:(1,-1)             */
/* State = post-collision populations, SoA f[q*nx*ny + y*nx + x].  Cell flags: 0 fluid,       */
/* 1 stationary wall, 2 moving wall (velocity uw).  periodic: bit0 x, bit1 y.                  */
/* ------------------------------------------------------------------------------------------ */
static const int CX9[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CY9[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int OPP9[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

#define D2Q9_IMPL(REAL, SUF)                                                                       \
    static const REAL W9_##SUF[9] = {(REAL)(4.0 / 9.0),  (REAL)(1.0 / 9.0),  (REAL)(1.0 / 9.0),   \
                                     (REAL)(1.0 / 9.0),  (REAL)(1.0 / 9.0),  (REAL)(1.0 / 36.0),  \
                                     (REAL)(1.0 / 36.0), (REAL)(1.0 / 36.0), (REAL)(1.0 / 36.0)}; \
                                                                                                   \
    /* streamed (pre-collision) populations of fluid cell (x,y) */                                 \
    static void d2q9_gather_##SUF(int nx, int ny, int periodic, const uint8_t *flags, REAL uwx,    \
                                  REAL uwy, const REAL *src, int x, int y, REAL fin[9]) {          \
        long N = (long)nx * ny, c = (long)y * nx + x;                                             \
        for (int j = 0; j < 9; ++j) {                                                              \
            int sx = x - CX9[j], sy = y - CY9[j];                                                  \
            if (periodic & 1) sx = (sx + nx) % nx;                                                 \
            if (periodic & 2) sy = (sy + ny) % ny;                                                 \
            int wall = 0;                                                                          \
            if (sx < 0 || sy < 0 || sx >= nx || sy >= ny)                                          \
                wall = 1;                                                                          \
            else if (flags[(long)sy * nx + sx] != 0)                                               \
                wall = flags[(long)sy * nx + sx] == 2 ? 2 : 1;                                     \
            if (!wall) {                                                                           \
                fin[j] = src[j * N + (long)sy * nx + sx];                                          \
            } else {                                                                               \
                REAL v = src[OPP9[j] * N + c];                                                     \
                if (wall == 2) v += (REAL)6 * W9_##SUF[j] * ((REAL)CX9[j] * uwx + (REAL)CY9[j] * uwy); \
                fin[j] = v;                                                                        \
            }                                                                                      \
        }                                                                                          \
    }                                                                                              \
                                                                                                   \
    int orc_d2q9_step_##SUF(int nx, int ny, int periodic, const uint8_t *flags, REAL tau, REAL fx, \
                            REAL fy, REAL uwx, REAL uwy, const REAL *src, REAL *dst) {             \
        long N = (long)nx * ny;                                                                    \
        REAL omega = (REAL)1 / tau;                                                                \
        REAL fpre = (REAL)1 - omega / (REAL)2;                                                     \
        _Pragma("omp parallel for schedule(static)") for (int y = 0; y < ny; ++y) {               \
            for (int x = 0; x < nx; ++x) {                                                         \
                long c = (long)y * nx + x;                                                         \
                if (flags[c] != 0) {                                                               \
                    for (int q = 0; q < 9; ++q) dst[q * N + c] = src[q * N + c];                   \
                    continue;                                                                      \
                }                                                                                  \
                REAL fin[9];                                                                       \
                d2q9_gather_##SUF(nx, ny, periodic, flags, uwx, uwy, src, x, y, fin);              \
                REAL rho = 0, mx = 0, my = 0;                                                      \
                for (int j = 0; j < 9; ++j) {                                                      \
                    rho += fin[j];                                                                 \
                    mx += fin[j] * (REAL)CX9[j];                                                   \
                    my += fin[j] * (REAL)CY9[j];                                                   \
                }                                                                                  \
                REAL ux = (mx + fx / (REAL)2) / rho, uy = (my + fy / (REAL)2) / rho;               \
                REAL usq = ux * ux + uy * uy;                                                      \
                for (int j = 0; j < 9; ++j) {                                                      \
                    REAL cu = (REAL)CX9[j] * ux + (REAL)CY9[j] * uy;                               \
                    REAL feq = W9_##SUF[j] * rho *                                                 \
                               ((REAL)1 + (REAL)3 * cu + (REAL)4.5 * cu * cu - (REAL)1.5 * usq);   \
                    REAL cf = (REAL)CX9[j] * fx + (REAL)CY9[j] * fy;                               \
                    REAL uf = ux * fx + uy * fy;                                                   \
                    REAL S = fpre * W9_##SUF[j] * ((REAL)3 * (cf - uf) + (REAL)9 * cu * cf);       \
                    dst[j * N + c] = fin[j] + omega * (feq - fin[j]) + S;                          \
                }                                                                                  \
            }                                                                                      \
        }                                                                                          \
        return 0;                                                                                  \
    }                                                                                              \
                                                                                                   \
    int orc_d2q9_run_##SUF(int nx, int ny, int periodic, const uint8_t *flags, REAL tau, REAL fx,  \
                           REAL fy, REAL uwx, REAL uwy, REAL *f, int nsteps) {                     \
        long N = (long)nx * ny;                                                                    \
        REAL *tmp = (REAL *)malloc(sizeof(REAL) * 9 * (size_t)N);                                 \
        if (!tmp) return -3;                                                                       \
        REAL *a = f, *b = tmp;                                                                     \
        for (int s = 0; s < nsteps; ++s) {                                                         \
            orc_d2q9_step_##SUF(nx, ny, periodic, flags, tau, fx, fy, uwx, uwy, a, b);             \
            REAL *t = a;                                                                           \
            a = b;                                                                                 \
            b = t;                                                                                 \
        }                                                                                          \
        if (a != f) memcpy(f, a, sizeof(REAL) * 9 * (size_t)N);                                    \
        free(tmp);                                                                                 \
        return 0;                                                                                  \
    }                                                                                              \
                                                                                                   \
    /* fields at the current time: density and velocity of the streamed populations, with the  */ \
    /* half-force shift; solid cells report rho = 1, u = 0                                       */ \
    int orc_d2q9_moments_##SUF(int nx, int ny, int periodic, const uint8_t *flags, REAL fx,       \
                               REAL fy, REAL uwx, REAL uwy, const REAL *f, REAL *rho_out,          \
                               REAL *ux_out, REAL *uy_out) {                                       \
        _Pragma("omp parallel for schedule(static)") for (int y = 0; y < ny; ++y) {               \
            for (int x = 0; x < nx; ++x) {                                                         \
                long c = (long)y * nx + x;                                                         \
                if (flags[c] != 0) {                                                               \
                    rho_out[c] = 1;                                                                \
                    ux_out[c] = 0;                                                                 \
                    uy_out[c] = 0;                                                                 \
                    continue;                                                                      \
                }                                                                                  \
                REAL fin[9];                                                                       \
                d2q9_gather_##SUF(nx, ny, periodic, flags, uwx, uwy, f, x, y, fin);                \
                REAL rho = 0, mx = 0, my = 0;                                                      \
                for (int j = 0; j < 9; ++j) {                                                      \
                    rho += fin[j];                                                                 \
                    mx += fin[j] * (REAL)CX9[j];                                                   \
                    my += fin[j] * (REAL)CY9[j];                                                   \
                }                                                                                  \
                rho_out[c] = rho;                                                                  \
                ux_out[c] = (mx + fx / (REAL)2) / rho;                                             \
                uy_out[c] = (my + fy / (REAL)2) / rho;                                             \
            }                                                                                      \
        }                                                                                          \
        return 0;                                                                                  \
    }                                                                                              \
                                                                                                   \
    /* f = feq(rho, u) everywhere (rho/ux/uy may be NULL: 1, 0, 0) */                              \
    int orc_d2q9_equilibrium_##SUF(int nx, int ny, const REAL *rho, const REAL *ux,                \
                                   const REAL *uy, REAL *f) {                                      \
        long N = (long)nx * ny;                                                                    \
        for (long c = 0; c < N; ++c) {                                                             \
            REAL r = rho ? rho[c] : (REAL)1, u = ux ? ux[c] : (REAL)0, v = uy ? uy[c] : (REAL)0;   \
            REAL usq = u * u + v * v;                                                              \
            for (int j = 0; j < 9; ++j) {                                                          \
                REAL cu = (REAL)CX9[j] * u + (REAL)CY9[j] * v;                                     \
                f[j * N + c] = W9_##SUF[j] * r *                                                   \
                               ((REAL)1 + (REAL)3 * cu + (REAL)4.5 * cu * cu - (REAL)1.5 * usq);   \
            }                                                                                      \
        }                                                                                          \
        return 0;                                                                                  \
    }                                                                                              \
                                                                                                   \
    /* mass and momentum of the stored populations over fluid cells, summed in double */          \
    int orc_d2q9_conservation_##SUF(int nx, int ny, const uint8_t *flags, const REAL *f,           \
                                    double out[3]) {                                               \
        long N = (long)nx * ny;                                                                    \
        double m = 0, px = 0, py = 0;                                                              \
        for (long c = 0; c < N; ++c) {                                                             \
            if (flags[c] != 0) continue;                                                           \
            for (int j = 0; j < 9; ++j) {                                                          \
                double v = (double)f[j * N + c];                                                   \
                m += v;                                                                            \
                px += v * CX9[j];                                                                  \
                py += v * CY9[j];                                                                  \
            }                                                                                      \
        }                                                                                          \
        out[0] = m;                                                                                \
        out[1] = px;                                                                               \
        out[2] = py;                                                                               \
        return 0;                                                                                  \
    }

D2Q9_IMPL(double, f64)
D2Q9_IMPL(float, f32)

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
