// The reference's simulation/include C++ API (Lattice, Model, FlowData, RunCudaFunctions, Constants,
// Utils, rotateVectorAroundAxis) implemented on the library's C ABI, mode LBM_D3Q27_REF.
//
//   Lattice         Lattice.cpp:22-477      one lbm_ctx per Lattice; the simulate* passes map to
//                                           lbm_apply, simulateLattice to one fused lbm_step
//   Model           Model.cpp:22-91         lbm_mesh_* (OBJ reader, point in mesh, reflection vector)
//   FlowCriterion   FlowCriterion.cu:3-17   host predicates, evaluated once per cell by setFlowData
//   RunCudaFunctions SimCalcFuncs.cu:218-249 the same passes on a lattice named by its LatticeData
//   Utils::compressInts Utils.cpp:9-37, CONSTANTS Constants.cpp:3-8
//
// Error behaviour follows the reference: failures are printed ("<method> failed: <reason>") and the
// call returns; retrieve_data returns nullptr on failure.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <set>
#include <sys/stat.h>

#include "Constants.h"
#include "FlowCriterion.cuh"
#include "FlowSurface.h"
#include "Geometry.h"
#include "Lattice.h"
#include "LatticePoint.h"
#include "Model.h"
#include "SimCalcFuncs.cuh"
#include "Utils.h"
#include "lbm_capi.h"

// ------------------------------------------------------------------ constants and small helpers
namespace CONSTANTS
{
    const float GEOMETRIC_TOLERANCE = 1e-6f;
    // population order of the reference's LatticePoint (Constants.cpp:6-7)
    const int DIRECTIONS[27][3] = {
        {0, 0, 0},   {-1, 0, 0},  {0, -1, 0},  {0, 0, -1},  {0, 0, 1},   {0, 1, 0},    {1, 0, 0},
        {-1, -1, 0}, {-1, 0, -1}, {-1, 0, 1},  {-1, 1, 0},  {0, -1, -1}, {0, -1, 1},   {0, 1, -1},
        {0, 1, 1},   {1, -1, 0},  {1, 0, -1},  {1, 0, 1},   {1, 1, 0},   {-1, -1, -1}, {-1, -1, 1},
        {-1, 1, -1}, {-1, 1, 1},  {1, -1, -1}, {1, -1, 1},  {1, 1, -1},  {1, 1, 1}};
    const int INVERSE_DIRECTIONS[27] = {0,  6,  5,  4,  3,  2,  1,  18, 17, 16, 15, 14, 13, 12,
                                        11, 10, 9,  8,  7,  26, 25, 24, 23, 22, 21, 20, 19};
}

namespace Utils
{
    unsigned int compressInts(int* array, const int num, const int bitLength)
    {
        unsigned int limit = 1;
        for (int b = 0; b < bitLength; ++b) limit *= 2;
        unsigned int out = 0;
        for (int i = 0; i + 1 < num; ++i)
            if ((unsigned int)array[i] < limit) out = (out | (unsigned int)array[i]) << 5;  // values at or above the limit are skipped
        if (num > 0 && (unsigned int)array[num - 1] < limit) out |= (unsigned int)array[num - 1];
        return out;
    }
}

namespace FlowCriterion
{
    bool testCriteria(int x, int y, int z) { return x == 1 && y == 1 && z == 1; }
    bool testPlaneCriteria(int x, int, int) { return x == 0; }

    bool (*ptestCriteria)(int, int, int) = &testCriteria;
    bool (*ptestPlaneCriteria)(int, int, int) = &testPlaneCriteria;
}

Point_3 rotateVectorAroundAxis(Point_3 axis, Point_3 vector, float angle)
{
    const float a[3] = {axis.x, axis.y, axis.z}, v[3] = {vector.x, vector.y, vector.z};
    float out[3];
    lbm_rotate_vector(a, v, angle, out);
    return Point_3(out[0], out[1], out[2]);
}

namespace {

// live lattices, so that the RunCudaFunctions launchers accept only handles of existing ones
std::mutex g_live_mu;
std::set<lbm_ctx*> g_live;

void report(const char* where, const char* why) { printf("%s failed: %s\n", where, why); }

bool file_exists(const std::string& path)
{
    struct stat st;
    return stat(path.c_str(), &st) == 0;
}

}  // namespace

// ------------------------------------------------------------------ Model
Model::~Model() { lbm_mesh_destroy(mesh); }

void Model::importModel(std::string filename)
{
    if (!file_exists(filename)) return;  // as the reference: the model stays as it was
    lbm_mesh* m = nullptr;
    if (lbm_mesh_load_obj(filename.c_str(), &m) != LBM_OK) {
        report("Model::importModel", lbm_last_error(nullptr));
        meshValid = false;
        return;
    }
    lbm_mesh_destroy(mesh);
    mesh = m;
    lbm_mesh_info info;
    lbm_mesh_get_info(mesh, &info);
    modelMesh.vertices = info.vertices;
    modelMesh.faces = info.faces;
    meshValid = info.valid != 0;
}

bool Model::isModelClosed()
{
    if (!mesh) return true;  // an empty mesh has no border edge
    lbm_mesh_info info;
    lbm_mesh_get_info(mesh, &info);
    return info.closed != 0;
}

bool Model::isPointInsideModel(Point_3 point)
{
    if (!meshValid || !mesh) return false;
    const float p[3] = {point.x, point.y, point.z};
    int32_t inside = 0;
    lbm_mesh_point_inside(mesh, p, &inside);
    return inside != 0;
}

BoundingBox Model::bounding_box()
{
    BoundingBox b;
    if (!mesh) return b;
    lbm_mesh_info info;
    lbm_mesh_get_info(mesh, &info);
    for (int k = 0; k < 3; ++k) b.lo[k] = info.bbox_min[k], b.hi[k] = info.bbox_max[k];
    return b;
}

Point_3 Model::reflectionVector(Point_3 point_1, Point_3 point_2)
{
    if (!mesh) return Point_3(0.0f, 0.0f, 0.0f);
    const float a[3] = {point_1.x, point_1.y, point_1.z}, b[3] = {point_2.x, point_2.y, point_2.z};
    float out[3];
    lbm_mesh_reflection_vector(mesh, a, b, out);
    return Point_3(out[0], out[1], out[2]);
}

// ------------------------------------------------------------------ Lattice
Lattice::Lattice(int x, int y, int z, dim3 blocks, dim3 threads, FluidData fluid, float spacing)
    : m_fluid(fluid),
      m_xResolution((unsigned short)x),
      m_yResolution((unsigned short)y),
      m_zResolution((unsigned short)z),
      m_latticeSpacing(spacing),
      m_threads(threads),
      m_blocks(blocks)
{
    lbm_desc d;
    lbm_desc_init(&d);
    d.mode = LBM_D3Q27_REF;
    d.dtype = LBM_F32;
    d.nx = x;
    d.ny = y;
    d.nz = z;
    d.tau = fluid.m_characteristicTimescale;
    d.order = LBM_ORDER_STREAM_COLLIDE;
    d.force_mode = LBM_FORCE_REFERENCE;
    if (ok(lbm_create(&d, &m_ctx), "Lattice::Lattice")) {
        std::lock_guard<std::mutex> g(g_live_mu);
        g_live.insert(m_ctx);
    }
}

Lattice::~Lattice()
{
    if (m_ctx) {
        std::lock_guard<std::mutex> g(g_live_mu);
        g_live.erase(m_ctx);
    }
    lbm_destroy(m_ctx);
    delete m_simModel;
}

bool Lattice::ok(int status, const char* where)
{
    if (status == LBM_OK) return true;
    m_error = std::string(where) + ": " + lbm_last_error(m_ctx);
    report(where, lbm_last_error(m_ctx));
    return false;
}

cudaPitchedPtr Lattice::getCudaDataPointer()
{
    return make_cudaPitchedPtr(m_ctx, 0, m_xResolution, m_yResolution);
}

void Lattice::load_data(LatticePoint* lattice_array)
{
    if (!lattice_array) {
        report("Lattice::load_data", "null array");
        return;
    }
    ok(lbm_load_aos(m_ctx, lattice_array, (int64_t)m_xResolution * m_yResolution * m_zResolution), "Lattice::load_data");
}

LatticePoint* Lattice::retrieve_data()
{
    const int64_t n = (int64_t)m_xResolution * m_yResolution * m_zResolution;
    LatticePoint* out = new LatticePoint[(size_t)n];
    if (!ok(lbm_retrieve_aos(m_ctx, out, n), "Lattice::retrieve_data")) {
        delete[] out;
        return nullptr;
    }
    for (size_t i = 0; i < m_reflectionCells.size(); ++i) out[m_reflectionCells[i]].reflections = &m_reflections[i];
    return out;
}

ReflectionData* Lattice::retrieve_reflection_data()
{
    if (!m_reflectionData) {
        report("Lattice::retrieve_reflection_data", "no ReflectionData set");
        return nullptr;
    }
    float f[3];
    if (ok(lbm_get_force(m_ctx, f), "Lattice::retrieve_reflection_data")) {
        m_reflectionData->x = f[0];
        m_reflectionData->y = f[1];
        m_reflectionData->z = f[2];
    }
    return m_reflectionData;
}

void Lattice::simulateStreaming() { ok(lbm_apply(m_ctx, LBM_OP_STREAM), "Lattice::simulateStreaming"); }

void Lattice::simulateCollision()
{
    if (ok(lbm_set_params(m_ctx, m_fluid.m_characteristicTimescale, nullptr, nullptr), "Lattice::simulateCollision"))
        ok(lbm_apply(m_ctx, LBM_OP_COLLIDE), "Lattice::simulateCollision");
}

void Lattice::simulateReflections() { ok(lbm_apply(m_ctx, LBM_OP_REFLECT), "Lattice::simulateReflections"); }

void Lattice::simulateFlow()
{
    if (m_flowData) ok(lbm_apply(m_ctx, LBM_OP_FLOW), "Lattice::simulateFlow");
}

void Lattice::simulateLattice()
{
    if (ok(lbm_set_order(m_ctx, LBM_ORDER_STREAM_COLLIDE), "Lattice::simulateLattice"))
        ok(lbm_step(m_ctx, 1), "Lattice::simulateLattice");
}

void Lattice::simulateSteps(int nsteps)
{
    if (ok(lbm_set_order(m_ctx, LBM_ORDER_CLI), "Lattice::simulateSteps")) ok(lbm_step(m_ctx, nsteps), "Lattice::simulateSteps");
}

std::vector<ReflectionData> Lattice::simulateStepsWithForce(int nsteps)
{
    std::vector<ReflectionData> out;
    if (nsteps <= 0 || !ok(lbm_set_order(m_ctx, LBM_ORDER_CLI), "Lattice::simulateStepsWithForce")) return out;
    std::vector<float> series((size_t)nsteps * 3);
    if (!ok(lbm_step_force_series(m_ctx, nsteps, series.data()), "Lattice::simulateStepsWithForce")) return out;
    out.resize((size_t)nsteps);
    for (int s = 0; s < nsteps; ++s) out[(size_t)s] = ReflectionData{series[3 * (size_t)s], series[3 * (size_t)s + 1], series[3 * (size_t)s + 2]};
    if (m_reflectionData) *m_reflectionData = out.back();
    return out;
}

void Lattice::refreshFlags(std::vector<unsigned char>& flags)
{
    flags.assign((size_t)m_xResolution * m_yResolution * m_zResolution, 0);
    ok(lbm_get_flags(m_ctx, flags.data()), "Lattice::flags");
}

void Lattice::insertModel(std::string filename)
{
    delete m_simModel;
    m_simModel = new Model();
    m_simModel->importModel(filename);
    if (!m_simModel->handle()) {
        report("Lattice::insertModel", ("cannot read " + filename).c_str());
        return;
    }
    std::vector<unsigned char> flags;
    refreshFlags(flags);
    int32_t applied = 0;
    if (!ok(lbm_mesh_rasterize(m_simModel->handle(), m_xResolution, m_yResolution, m_zResolution, m_latticeSpacing,
                               flags.data(), &applied), "Lattice::insertModel"))
        return;
    if (applied) ok(lbm_set_flags(m_ctx, flags.data()), "Lattice::insertModel");
}

std::array<std::pair<float, int>, 27> Lattice::distributeVector(Point_3 vector)
{
    const float v[3] = {vector.x, vector.y, vector.z};
    float score[27];
    int32_t dirs[27];
    lbm_distribute_vector(v, score, dirs);
    std::array<std::pair<float, int>, 27> out;
    for (int i = 0; i < 27; ++i) out[(size_t)i] = {score[i], (int)dirs[i]};
    return out;
}

void Lattice::preProcessModel()
{
    if (!m_simModel || !m_simModel->handle()) return;
    std::vector<unsigned char> flags;
    refreshFlags(flags);
    int64_t count = 0;
    lbm_mesh* mesh = m_simModel->handle();
    if (!ok(lbm_mesh_reflection_tables(mesh, m_xResolution, m_yResolution, m_zResolution, m_latticeSpacing, flags.data(), 0,
                                       nullptr, nullptr, &count), "Lattice::preProcessModel"))
        return;
    std::vector<int> cells((size_t)count);
    std::vector<ReflectionValues> recs((size_t)count);
    if (count > 0 && !ok(lbm_mesh_reflection_tables(mesh, m_xResolution, m_yResolution, m_zResolution, m_latticeSpacing,
                                                    flags.data(), count, cells.data(), recs.data(), &count),
                         "Lattice::preProcessModel"))
        return;
    if (!ok(lbm_set_flags(m_ctx, flags.data()), "Lattice::preProcessModel")) return;
    if (!ok(lbm_set_reflection_tables(m_ctx, count, cells.data(), recs.data()), "Lattice::preProcessModel")) return;
    m_reflectionCells.swap(cells);
    m_reflections.swap(recs);
}

void Lattice::setFlowData(FlowData* flowData)
{
    m_flowData = flowData;
    if (!flowData || !flowData->pointCriterion) {
        report("Lattice::setFlowData", "no flow criterion");
        return;
    }
    std::vector<unsigned char> mask((size_t)m_xResolution * m_yResolution * m_zResolution);
    size_t c = 0;
    for (int x = 0; x < m_xResolution; ++x)
        for (int y = 0; y < m_yResolution; ++y)
            for (int z = 0; z < m_zResolution; ++z) mask[c++] = flowData->pointCriterion(x, y, z) ? 1 : 0;
    ok(lbm_set_flow(m_ctx, mask.data(), flowData->inducedFlow.particle_distribution), "Lattice::setFlowData");
}

void Lattice::setReflectionData(ReflectionData* reflection)
{
    m_reflectionData = reflection;
    if (!reflection) {
        ok(lbm_set_force(m_ctx, nullptr, 0), "Lattice::setReflectionData");
        return;
    }
    const float in[3] = {reflection->x, reflection->y, reflection->z};
    ok(lbm_set_force(m_ctx, in, 1), "Lattice::setReflectionData");
}

// 81 slots of 5 bits, six to an int: slot `index` at bits 5 * (index % 6) of word index / 6
void Lattice::setReflectionDirection(LatticePoint* point, const int index, const unsigned int value)
{
    const unsigned int shift = 5u * (unsigned int)(index % 6);
    unsigned int word = (unsigned int)point->reflections->reflection_directions[index / 6];
    word = (word & ~(31u << shift)) | (value << shift);
    point->reflections->reflection_directions[index / 6] = (int)word;
}

int Lattice::getReflectionDirection(LatticePoint* point, const int index)
{
    const unsigned int shift = 5u * (unsigned int)(index % 6);
    return (int)(((unsigned int)point->reflections->reflection_directions[index / 6] >> shift) & 31u);
}

// ------------------------------------------------------------------ RunCudaFunctions
namespace {

lbm_ctx* lattice_of(const LatticeData& lattice, const char* where)
{
    lbm_ctx* ctx = static_cast<lbm_ctx*>(lattice.latticePtr.ptr);
    std::lock_guard<std::mutex> g(g_live_mu);
    if (!ctx || !g_live.count(ctx)) {
        report(where, "LatticeData does not name a live Lattice (use Lattice::getCudaDataPointer())");
        return nullptr;
    }
    return ctx;
}

void run(lbm_ctx* ctx, int status, const char* where)
{
    if (ctx && status != LBM_OK) report(where, lbm_last_error(ctx));
}

}  // namespace

namespace RunCudaFunctions
{
    void run_calculate_streaming(dim3, dim3, LatticeData lattice, LatticeData)
    {
        const char* w = "run_calculate_streaming";
        if (lbm_ctx* c = lattice_of(lattice, w)) run(c, lbm_apply(c, LBM_OP_STREAM), w);
    }

    void run_calculate_collision(dim3, dim3, LatticeData lattice, float timescale)
    {
        const char* w = "run_calculate_collision";
        if (lbm_ctx* c = lattice_of(lattice, w)) {
            const int st = lbm_set_params(c, timescale, nullptr, nullptr);
            run(c, st == LBM_OK ? lbm_apply(c, LBM_OP_COLLIDE) : st, w);
        }
    }

    void run_calculate_reflections(dim3, dim3, LatticeData lattice, LatticeData)
    {
        const char* w = "run_calculate_reflections";
        if (lbm_ctx* c = lattice_of(lattice, w)) {
            // the plain pass adds no force: pause accumulation around it
            const int32_t was = lbm_force_accumulation(c);
            int st = was ? lbm_set_force_accumulation(c, 0) : LBM_OK;
            if (st == LBM_OK) st = lbm_apply(c, LBM_OP_REFLECT);
            if (was) {
                const int st2 = lbm_set_force_accumulation(c, 1);
                if (st == LBM_OK) st = st2;
            }
            run(c, st, w);
        }
    }

    void run_calculate_reflections_data(dim3, dim3, LatticeData lattice, LatticeData, ReflectionData* reflection)
    {
        const char* w = "run_calculate_reflections_data";
        lbm_ctx* c = lattice_of(lattice, w);
        if (!c) return;
        if (!reflection) {
            report(w, "null ReflectionData");
            return;
        }
        // The reference passes the device copy that Lattice::setReflectionData made with cudaMalloc
        // (Lattice.cpp:58, 192); a host object works too.  A device object is read and written back
        // with cudaMemcpy, as Lattice::retrieve_reflection_data reads it (Lattice.cpp:440).
        cudaPointerAttributes attr{};
        bool on_device = false;
        if (cudaPointerGetAttributes(&attr, reflection) == cudaSuccess)
            on_device = attr.type == cudaMemoryTypeDevice;
        else
            cudaGetLastError();  // an unregistered host pointer: clear the error the query left
        ReflectionData value{};
        if (on_device) {
            if (cudaMemcpy(&value, reflection, sizeof(ReflectionData), cudaMemcpyDeviceToHost) != cudaSuccess) {
                report(w, cudaGetErrorString(cudaGetLastError()));
                return;
            }
        } else {
            value = *reflection;
        }
        // the pass adds its force to the object; the lattice's own accumulation state is restored after
        const int32_t was = lbm_force_accumulation(c);
        float keep[3] = {0.0f, 0.0f, 0.0f};
        const float in[3] = {value.x, value.y, value.z};
        float out[3];
        int st = lbm_get_force(c, keep);
        if (st == LBM_OK) st = lbm_set_force(c, in, 1);
        if (st == LBM_OK) st = lbm_apply(c, LBM_OP_REFLECT);
        if (st == LBM_OK) st = lbm_get_force(c, out);
        if (st == LBM_OK) st = lbm_set_force(c, keep, was);
        run(c, st, w);
        if (st != LBM_OK) return;
        value.x = out[0];
        value.y = out[1];
        value.z = out[2];
        if (!on_device) {
            *reflection = value;
        } else if (cudaMemcpy(reflection, &value, sizeof(ReflectionData), cudaMemcpyHostToDevice) != cudaSuccess) {
            report(w, cudaGetErrorString(cudaGetLastError()));
        }
    }

    void run_prime_points(dim3, dim3, LatticeData lattice) { lattice_of(lattice, "run_prime_points"); }

    void run_generate_flow(dim3, dim3, LatticeData lattice, FlowData* flowData)
    {
        const char* w = "run_generate_flow";
        lbm_ctx* c = lattice_of(lattice, w);
        if (!c) return;
        if (!flowData || !flowData->pointCriterion) {
            report(w, "no flow criterion");
            return;
        }
        lbm_info info;
        if (lbm_get_info(c, &info) != LBM_OK) return run(c, LBM_ERR_STATE, w);
        const int X = (int)lattice.latticeDimensions.x, Y = (int)lattice.latticeDimensions.y,
                  Z = (int)lattice.latticeDimensions.z;
        if ((int64_t)X * Y * Z != info.cells) {
            report(w, "LatticeData dimensions do not match the lattice");
            return;
        }
        std::vector<unsigned char> mask((size_t)info.cells);
        size_t i = 0;
        for (int x = 0; x < X; ++x)
            for (int y = 0; y < Y; ++y)
                for (int z = 0; z < Z; ++z) mask[i++] = flowData->pointCriterion(x, y, z) ? 1 : 0;
        int st = lbm_set_flow(c, mask.data(), flowData->inducedFlow.particle_distribution);
        if (st == LBM_OK) st = lbm_apply(c, LBM_OP_FLOW);
        run(c, st, w);
    }
}
