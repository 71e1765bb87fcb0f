// ref_harness.cpp -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// Runs the reference's own CUDA kernels (simulation/source/SimCalcFuncs.cu and FlowCriterion.cu,
// compiled from the reference's sources into oracle/_ref/ref_kernels.cubin by oracle/refkern.py)
// on seeded inputs, so that the GPU library can be compared with the reference itself.
//
// The kernels are loaded with the CUDA driver API and launched in the orders of the reference's
// Lattice class (simulation/source/Lattice.cpp): simulateStreaming (:115-154: copy the lattice to a
// temporary, stream into it, swap), simulateReflections (:163-210: same copy + swap), simulateCollision
// (:156-161, in place) and simulateFlow (:212-220, in place).  Lattice.cpp itself needs CGAL and is
// not built; this harness replaces its memory handling with one fixed pair of buffers.
//
// Layout: the reference addresses cell (x, y, z) at slice x, row y, element z of a pitched array
// (SimCalcFuncs.cu:32-50).  The harness uses pitch = Z records and slice pitch = Y*Z records, so the
// device record index equals the host index z + Z*(y + Y*x) for any X, Y, Z.  Launch: blocks of
// (tx, ty, tz) threads that tile the lattice exactly, as the unguarded kernels need (checked).
#include <cuda.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct ReflectionValues {  // LatticePoint.h:3-7
    int reflection_directions[14];
    float reflection_weight[81];
};
struct LatticePoint {  // LatticePoint.h:9-17
    int x, y, z;
    float particle_distribution[27];
    bool isReflected;
    bool isInternal;
    ReflectionValues *reflections;
    ReflectionValues *d_reflections;
};
struct LatticeData {  // Lattice.h:15-22
    cudaPitchedPtr latticePtr;
    dim3 latticeDimensions;
};
struct ReflectionData {  // Lattice.h:33-38
    float x, y, z;
};
struct FlowData {  // FlowSurface.h:9-46
    LatticePoint inducedFlow;
    bool (*pointCriterion)(int, int, int);
    int val;
};
static_assert(sizeof(LatticePoint) == 144, "LatticePoint layout");
static_assert(sizeof(ReflectionValues) == 380, "ReflectionValues layout");

std::string g_err;
double g_last_seconds = 0.0;
CUmodule g_mod = nullptr;
CUfunction g_stream, g_collide, g_reflect, g_flow, g_prime;
CUdeviceptr g_crit_point = 0, g_crit_plane = 0;
CUcontext g_ctx = nullptr;

int fail(const std::string &m) {
    g_err = m;
    return -1;
}

#define CU(call)                                                                     \
    do {                                                                             \
        CUresult r_ = (call);                                                        \
        if (r_ != CUDA_SUCCESS) {                                                    \
            const char *s_ = nullptr;                                                \
            cuGetErrorString(r_, &s_);                                               \
            return fail(std::string(#call) + ": " + (s_ ? s_ : "?"));               \
        }                                                                            \
    } while (0)

int g_t[3] = {1, 1, 1};

int launch(CUfunction fn, int X, int Y, int Z, void **args) {
    CU(cuLaunchKernel(fn, X / g_t[0], Y / g_t[1], Z / g_t[2], g_t[0], g_t[1], g_t[2], 0, nullptr, args, nullptr));
    CU(cuCtxSynchronize());
    return 0;
}

LatticeData data_of(CUdeviceptr p, int X, int Y, int Z) {
    LatticeData d;
    d.latticePtr.ptr = reinterpret_cast<void *>(p);
    d.latticePtr.pitch = sizeof(LatticePoint) * (size_t)Z;
    d.latticePtr.xsize = (size_t)Z;
    d.latticePtr.ysize = (size_t)Y;
    d.latticeDimensions = dim3(X, Y, Z);
    return d;
}

int refl_dir(const ReflectionValues &r, int s) {
    return (int)(((unsigned)r.reflection_directions[s / 6] >> (5 * (s % 6))) & 31u);
}

}  // namespace

extern "C" {

const char *rk_error() { return g_err.c_str(); }

// seconds of the last rk_run's step loop (launches, temporary copies and synchronisations; not the
// set-up, upload or download)
double rk_last_seconds() { return g_last_seconds; }

int rk_init(const char *cubin_path) {
    if (g_mod) return 0;
    CU(cuInit(0));
    CUdevice dev;
    CU(cuDeviceGet(&dev, 0));
    CU(cuDevicePrimaryCtxRetain(&g_ctx, dev));
    CU(cuCtxSetCurrent(g_ctx));
    CU(cuModuleLoad(&g_mod, cubin_path));
    CU(cuModuleGetFunction(&g_stream, g_mod, "_ZN13CudaFunctions19calculate_streamingE11LatticeDataS0_"));
    CU(cuModuleGetFunction(&g_collide, g_mod, "_ZN13CudaFunctions19calculate_collisionE11LatticeDataf"));
    CU(cuModuleGetFunction(&g_reflect, g_mod, "_ZN13CudaFunctions21calculate_reflectionsE11LatticeDataS0_P14ReflectionData"));
    CU(cuModuleGetFunction(&g_flow, g_mod, "_ZN13CudaFunctions13generate_flowE11LatticeDataP8FlowData"));
    CU(cuModuleGetFunction(&g_prime, g_mod, "_ZN13CudaFunctions12prime_pointsE11LatticeData"));
    size_t sz = 0;
    CU(cuModuleGetGlobal(&g_crit_point, &sz, g_mod, "_ZN13FlowCriterion13ptestCriteriaE"));
    CU(cuModuleGetGlobal(&g_crit_plane, &sz, g_mod, "_ZN13FlowCriterion18ptestPlaneCriteriaE"));
    return 0;
}

// Run `nsteps` repetitions of the pass sequence `ops` (characters S stream, R reflect, C collide,
// F flow) on the X*Y*Z records in `points` (host, updated in place).  Reflection records
// `tab_records[i]` belong to cell `tab_cells[i]`.  flow_criterion: 0 none, 1 the point (1,1,1)
// (FlowCriterion.cu:5-8), 2 the plane x = 0 (FlowCriterion.cu:10-13).  `force` (nullable) is the
// ReflectionData start value and receives the final sum; with a force, every table slot must be
// below 27 (the reference's force reads DIRECTIONS/SPLIT at the slot index).  threads[3]: block
// shape, each dividing its dimension.
int rk_run(int X, int Y, int Z, void *points, const int32_t *tab_cells, const void *tab_records, int ntab, float tau,
           const char *ops, int nsteps, int flow_criterion, const float *induced, float *force, const int *threads) {
    if (!g_mod) return fail("rk_init not called");
    if (X < 1 || Y < 1 || Z < 1) return fail("unsupported dimensions");
    const int tx = threads ? threads[0] : 1, ty = threads ? threads[1] : 1, tz = threads ? threads[2] : 1;
    if (tx < 1 || ty < 1 || tz < 1 || tz > 64 || tx * ty * tz > 1024 || X % tx || Y % ty || Z % tz)
        return fail("block shape must tile the lattice exactly (and tz <= 64, tx*ty*tz <= 1024)");
    if (X / tx > 2147483647 || Y / ty > 65535 || Z / tz > 65535) return fail("grid too large");
    g_t[0] = tx;
    g_t[1] = ty;
    g_t[2] = tz;
    CU(cuCtxSetCurrent(g_ctx));
    const size_t n = (size_t)X * Y * Z;
    const ReflectionValues *recs = static_cast<const ReflectionValues *>(tab_records);
    for (int i = 0; i < ntab; ++i) {
        if (tab_cells[i] < 0 || (size_t)tab_cells[i] >= n) return fail("table cell out of range");
        for (int s = 1; s < 81; ++s) {
            const int d = refl_dir(recs[i], s);
            if (d > 26) return fail("table direction out of range");
            if (force && d != 0 && s >= 27) return fail("force with a slot >= 27");
        }
    }
    std::vector<LatticePoint> host(n);
    std::memcpy(host.data(), points, n * sizeof(LatticePoint));
    CUdeviceptr a = 0, b = 0, drec = 0, dref = 0, dflow = 0;
    CU(cuMemAlloc(&a, n * sizeof(LatticePoint)));
    CU(cuMemAlloc(&b, n * sizeof(LatticePoint)));
    if (ntab) CU(cuMemAlloc(&drec, ntab * sizeof(ReflectionValues)));
    for (size_t c = 0; c < n; ++c) {
        host[c].reflections = nullptr;
        host[c].d_reflections = nullptr;
    }
    for (int i = 0; i < ntab; ++i)
        host[tab_cells[i]].d_reflections = reinterpret_cast<ReflectionValues *>(drec + i * sizeof(ReflectionValues));
    // the reference dereferences d_reflections of every reflected cell (SimCalcFuncs.cu:162-166)
    for (size_t c = 0; c < n; ++c)
        if (host[c].isReflected && !host[c].d_reflections) {
            cuMemFree(a);
            cuMemFree(b);
            if (drec) cuMemFree(drec);
            return fail("reflected cell " + std::to_string(c) + " has no reflection table");
        }
    int rc = 0;
    auto body = [&]() -> int {
        if (ntab) CU(cuMemcpyHtoD(drec, recs, ntab * sizeof(ReflectionValues)));
        CU(cuMemcpyHtoD(a, host.data(), n * sizeof(LatticePoint)));
        if (force) {
            CU(cuMemAlloc(&dref, sizeof(ReflectionData)));
            CU(cuMemcpyHtoD(dref, force, sizeof(ReflectionData)));
        }
        if (flow_criterion) {
            FlowData fd;
            std::memset(&fd, 0, sizeof(fd));
            for (int q = 0; q < 27; ++q) fd.inducedFlow.particle_distribution[q] = induced[q];
            CU(cuMemcpyDtoH(&fd.pointCriterion, flow_criterion == 1 ? g_crit_point : g_crit_plane, sizeof(void *)));
            fd.val = 1;
            CU(cuMemAlloc(&dflow, sizeof(FlowData)));
            CU(cuMemcpyHtoD(dflow, &fd, sizeof(FlowData)));
        }
        LatticeData la = data_of(a, X, Y, Z), lb = data_of(b, X, Y, Z);
        void *pargs[] = {&la};
        if (launch(g_prime, X, Y, Z, pargs)) return -1;  // RunCudaFunctions::run_prime_points
        const auto t_start = std::chrono::steady_clock::now();
        struct StepTimer {  // wall time of the step loop (every launch above and below synchronises)
            std::chrono::steady_clock::time_point t0;
            ~StepTimer() { g_last_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
        } timer{t_start};
        for (int step = 0; step < nsteps; ++step) {
            for (const char *o = ops; *o; ++o) {
                la = data_of(a, X, Y, Z);
                lb = data_of(b, X, Y, Z);
                if (*o == 'S' || *o == 'R') {
                    CU(cuMemcpyDtoD(b, a, n * sizeof(LatticePoint)));  // temporary copy
                    if (*o == 'S') {
                        void *args[] = {&la, &lb};
                        if (launch(g_stream, X, Y, Z, args)) return -1;
                    } else {
                        void *rp = reinterpret_cast<void *>(dref);
                        void *args[] = {&la, &lb, &rp};
                        if (launch(g_reflect, X, Y, Z, args)) return -1;
                    }
                    std::swap(a, b);
                } else if (*o == 'C') {
                    float t = tau;
                    void *args[] = {&la, &t};
                    if (launch(g_collide, X, Y, Z, args)) return -1;
                } else if (*o == 'F') {
                    if (dflow) {
                        void *fp = reinterpret_cast<void *>(dflow);
                        void *args[] = {&la, &fp};
                        if (launch(g_flow, X, Y, Z, args)) return -1;
                    }
                } else {
                    return fail(std::string("unknown pass '") + *o + "'");
                }
            }
        }
        CU(cuMemcpyDtoH(host.data(), a, n * sizeof(LatticePoint)));
        if (force) CU(cuMemcpyDtoH(force, dref, sizeof(ReflectionData)));
        return 0;
    };
    rc = body();
    if (a) cuMemFree(a);
    if (b) cuMemFree(b);
    if (drec) cuMemFree(drec);
    if (dref) cuMemFree(dref);
    if (dflow) cuMemFree(dflow);
    if (rc == 0) {
        for (size_t c = 0; c < n; ++c) {
            host[c].reflections = nullptr;
            host[c].d_reflections = nullptr;
        }
        std::memcpy(points, host.data(), n * sizeof(LatticePoint));
    }
    return rc;
}

}  // extern "C"
