// The reference's GoogleTest cases (test/CalculationsTest.cpp, CoordinatesTest.cpp, ModelTest.cpp,
// GeometryTest.cpp) rewritten against the compatibility layer (latticeboltzmanncuda_gb300/compat),
// i.e. the reference's own C++ API on this library.  GoogleTest is not available, so the program
// prints what each reference assertion checks, one JSON object per line:
//   {"test": "<suite>.<case>", "line": <line of the reference assertion>, "got": <value>}
//   {"test": ..., "line": ..., "mismatches": <count>}   for assertions inside loops
// and tests/test_compat_layer.py compares them with the expected values in tests/golden/.
//
// usage: compat_tests <dir with the test meshes as OBJ files> [--host-only]
// --host-only runs the cases that need no GPU (Model, Geometry, compressInts, distributeVector).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "Constants.h"
#include "FlowCriterion.cuh"
#include "FlowSurface.h"
#include "Geometry.h"
#include "Lattice.h"
#include "LatticePoint.h"
#include "Model.h"
#include "SimCalcFuncs.cuh"
#include "Utils.h"

static std::string g_dir;

static void got(const char* test, int line, double v) { printf("{\"test\": \"%s\", \"line\": %d, \"got\": %.9g}\n", test, line, v); }
static void mismatches(const char* test, int line, long n) { printf("{\"test\": \"%s\", \"line\": %d, \"mismatches\": %ld}\n", test, line, n); }
static std::string mesh(const char* name) { return g_dir + "/" + name; }

// The reference's tests load `new LatticePoint[n]` without initialising it and rely on fresh heap
// memory reading as zero; here the arrays are zeroed explicitly.
static LatticePoint* zeroed(size_t n)
{
    LatticePoint* a = new LatticePoint[n];
    memset(static_cast<void*>(a), 0, sizeof(LatticePoint) * n);
    return a;
}

static int at(Lattice& l, int x, int y, int z)
{
    dim3 d = l.getDimensions();
    return z + (y * d.z) + (x * d.z * d.y);
}

// ------------------------------------------------------------------ CalculationsTest
static void TestStreaming()
{
    dim3 threads(1, 2, 1), blocks(1, 1, 1);
    Lattice lattice(1, 2, 1, blocks, threads, FluidData(1.0, 1.0), 0.1);
    LatticeData data(lattice.getCudaDataPointer(), lattice.getDimensions());
    LatticePoint* a = zeroed(2);
    a[0].particle_distribution[5] = 2.0;
    lattice.load_data(a);
    RunCudaFunctions::run_prime_points(blocks, threads, data);
    lattice.simulateStreaming();
    delete[] a;
    a = lattice.retrieve_data();
    got("CalculationsTest.TestStreaming", 44, a[1].particle_distribution[5]);
    delete[] a;
}

static void TestCollision()
{
    dim3 threads(1, 1, 1), blocks(1, 1, 1);
    Lattice lattice(1, 1, 1, blocks, threads, FluidData(1.0, 1.0), 0.1);
    LatticePoint* a = zeroed(1);
    a[0].particle_distribution[0] = 2.0;
    lattice.load_data(a);
    lattice.simulateCollision();
    delete[] a;
    a = lattice.retrieve_data();
    got("CalculationsTest.TestCollision", 72, a[0].particle_distribution[0]);
    got("CalculationsTest.TestCollision", 73, a[0].particle_distribution[1]);
    got("CalculationsTest.TestCollision", 74, a[0].particle_distribution[2]);
    delete[] a;
}

static void TestFull()
{
    dim3 threads(1, 2, 1), blocks(1, 1, 1);
    Lattice lattice(1, 2, 1, blocks, threads, FluidData(1.0, 1.0), 0.1);
    LatticePoint* a = zeroed(2);
    a[0].particle_distribution[5] = 2.0;
    lattice.load_data(a);
    lattice.simulateLattice();
    delete[] a;
    a = lattice.retrieve_data();
    got("CalculationsTest.TestFull", 102, a[1].particle_distribution[0]);
    got("CalculationsTest.TestFull", 103, a[1].particle_distribution[1]);
    got("CalculationsTest.TestFull", 104, a[1].particle_distribution[2]);
    delete[] a;
}

static void TestReflections(bool withData)
{
    const char* name = withData ? "CalculationsTest.TestReflectionsData" : "CalculationsTest.TestReflections";
    dim3 threads(3, 3, 3), blocks(1, 1, 1);
    Lattice lattice(3, 3, 3, blocks, threads, FluidData(1.0, 1.0), 0.5);
    LatticeData data(lattice.getCudaDataPointer(), lattice.getDimensions());
    lattice.insertModel(mesh("cube_angled.obj"));
    lattice.preProcessModel();
    LatticePoint* a = lattice.retrieve_data();
    a[at(lattice, 1, 1, 1)].particle_distribution[1] = 1.0;
    lattice.load_data(a);
    delete[] a;
    ReflectionData* reflection = new ReflectionData;
    if (withData) lattice.setReflectionData(reflection);
    RunCudaFunctions::run_prime_points(blocks, threads, data);
    lattice.simulateReflections();
    a = lattice.retrieve_data();
    const int base = withData ? 186 : 141;
    got(name, base + 0, a[at(lattice, 2, 1, 2)].particle_distribution[17]);
    got(name, base + 1, a[at(lattice, 1, 1, 2)].particle_distribution[4]);
    got(name, base + 2, a[at(lattice, 2, 2, 2)].particle_distribution[26]);
    got(name, base + 4, a[at(lattice, 1, 1, 1)].particle_distribution[1]);
    delete[] a;
    if (withData) {
        reflection = lattice.retrieve_reflection_data();
        got(name, 194, reflection->x);
        got(name, 195, reflection->y);
        got(name, 196, reflection->z);
    }
    delete reflection;
}

// TestReflectionsData with the launcher called as Lattice::simulateReflections calls it
// (Lattice.cpp:192): the ReflectionData is the device copy that Lattice::allocateReflectionData makes
// with cudaMalloc (Lattice.cpp:58), read back with cudaMemcpy as retrieve_reflection_data does
// (Lattice.cpp:440).
static void TestReflectionsDeviceData()
{
    const char* name = "CalculationsTest.TestReflectionsData";
    dim3 threads(3, 3, 3), blocks(1, 1, 1);
    Lattice lattice(3, 3, 3, blocks, threads, FluidData(1.0, 1.0), 0.5);
    LatticeData data(lattice.getCudaDataPointer(), lattice.getDimensions());
    lattice.insertModel(mesh("cube_angled.obj"));
    lattice.preProcessModel();
    LatticePoint* a = lattice.retrieve_data();
    a[at(lattice, 1, 1, 1)].particle_distribution[1] = 1.0;
    lattice.load_data(a);
    delete[] a;
    ReflectionData start;
    ReflectionData* d_reflection = nullptr;
    if (cudaMalloc(&d_reflection, sizeof(ReflectionData)) != cudaSuccess ||
        cudaMemcpy(d_reflection, &start, sizeof(ReflectionData), cudaMemcpyHostToDevice) != cudaSuccess) {
        fprintf(stderr, "cudaMalloc / cudaMemcpy of the ReflectionData failed\n");
        return;
    }
    RunCudaFunctions::run_prime_points(blocks, threads, data);
    RunCudaFunctions::run_calculate_reflections_data(blocks, threads, data, data, d_reflection);
    a = lattice.retrieve_data();
    got(name, 186, a[at(lattice, 2, 1, 2)].particle_distribution[17]);
    got(name, 187, a[at(lattice, 1, 1, 2)].particle_distribution[4]);
    got(name, 188, a[at(lattice, 2, 2, 2)].particle_distribution[26]);
    got(name, 190, a[at(lattice, 1, 1, 1)].particle_distribution[1]);
    delete[] a;
    ReflectionData back;
    if (cudaMemcpy(&back, d_reflection, sizeof(ReflectionData), cudaMemcpyDeviceToHost) != cudaSuccess) {
        fprintf(stderr, "cudaMemcpy of the ReflectionData failed\n");
        cudaFree(d_reflection);
        return;
    }
    cudaFree(d_reflection);
    got(name, 194, back.x);
    got(name, 195, back.y);
    got(name, 196, back.z);
}

static void TestFlowGeneration(bool plane)
{
    dim3 threads(3, 3, 3), blocks(1, 1, 1);
    Lattice lattice(3, 3, 3, blocks, threads, FluidData(1.0, 1.0), 0.5);
    LatticeData data(lattice.getCudaDataPointer(), lattice.getDimensions());
    LatticePoint* a = zeroed(27);
    lattice.load_data(a);
    delete[] a;
    RunCudaFunctions::run_prime_points(blocks, threads, data);
    LatticePoint flowRef;
    flowRef.particle_distribution[0] = 1.0;
    FlowData* flow = new FlowData(plane ? &FlowCriterion::ptestPlaneCriteria : &FlowCriterion::ptestCriteria, flowRef);
    lattice.setFlowData(flow);
    lattice.simulateFlow();
    a = lattice.retrieve_data();
    if (!plane) {
        got("CalculationsTest.TestFlowGeneration", 232, a[at(lattice, 1, 1, 1)].particle_distribution[0]);
        got("CalculationsTest.TestFlowGeneration", 233, a[at(lattice, 0, 0, 0)].particle_distribution[0]);
    } else {
        for (int y = 0; y < 3; ++y)
            for (int z = 0; z < 3; ++z) {
                got("CalculationsTest.TestPlaneFlowGeneration", 273, a[at(lattice, 0, y, z)].particle_distribution[0]);
                got("CalculationsTest.TestPlaneFlowGeneration", 274, a[at(lattice, 1, y, z)].particle_distribution[0]);
            }
    }
    delete[] a;
    delete flow;
}

static void CompressionTest()
{
    int test_array[6] = {1, 2, 3, 4, 5, 6};
    got("CalculationsTest.CompressionTest", 283, Utils::compressInts(test_array, 6, 5));
}

// ------------------------------------------------------------------ CoordinatesTest
static void TestCoordsMatch()
{
    dim3 threads(10, 10, 10), blocks(10, 10, 10);
    Lattice lattice(100, 100, 100, blocks, threads, FluidData(1.0, 1.0), 0.1);
    LatticePoint* a = zeroed(100 * 100 * 100);
    int counter = 0;
    for (int x = 0; x < 100; ++x)
        for (int y = 0; y < 100; ++y)
            for (int z = 0; z < 100; ++z) {
                a[counter].x = x;
                a[counter].y = y;
                a[counter].z = z;
                ++counter;
            }
    lattice.load_data(a);
    delete[] a;
    a = lattice.retrieve_data();
    long bad[3] = {0, 0, 0};
    for (int x = 0; x < 100; ++x)
        for (int y = 0; y < 100; ++y)
            for (int z = 0; z < 100; ++z) {
                const LatticePoint& p = a[z + (y * 100) + (x * 10000)];
                bad[0] += p.x != x;
                bad[1] += p.y != y;
                bad[2] += p.z != z;
            }
    mismatches("CoordinatesTest.TestCoordsMatch", 80, bad[0]);
    mismatches("CoordinatesTest.TestCoordsMatch", 81, bad[1]);
    mismatches("CoordinatesTest.TestCoordsMatch", 82, bad[2]);
    delete[] a;
}

static void TestCoordinatesWithModel()
{
    dim3 threads(1, 1, 1), blocks(10, 10, 10);
    Lattice lattice(10, 10, 10, blocks, threads, FluidData(1.0, 1.0), 0.1);
    LatticePoint* a = zeroed(10 * 10 * 10);
    lattice.load_data(a);
    delete[] a;
    lattice.insertModel(mesh("compat_cube.obj"));
    a = lattice.retrieve_data();
    long outside = 0, inside = 0;
    for (int y = 0; y < 10; ++y)
        for (int x = 0; x < 10; ++x) outside += a[(10 * y) + x].isInternal ? 1 : 0;
    for (int y = 1; y < 9; ++y)
        for (int x = 1; x < 9; ++x) inside += a[500 + (10 * y) + x].isInternal ? 0 : 1;
    mismatches("CoordinatesTest.TestCoordinatesWithModel", 158, outside);
    mismatches("CoordinatesTest.TestCoordinatesWithModel", 166, inside);
    delete[] a;
}

static void TestDistributeVector()
{
    dim3 threads(1, 1, 1), blocks(1, 1, 1);
    Lattice lattice(1, 1, 1, blocks, threads, FluidData(1.0, 1.0), 0.1);
    std::array<std::pair<float, int>, 27> r = lattice.distributeVector(Point_3(1.0, 0.1, 0.1));
    const float norm = r[0].first + r[1].first + r[2].first;
    for (int k = 0; k < 3; ++k) {
        got("CoordinatesTest.TestDistributeVector", 192 + k, r[k].first / norm);
        got("CoordinatesTest.TestDistributeVector", 195 + k, r[k].second);
    }
}

static void TestReflection()
{
    dim3 threads(3, 3, 3), blocks(1, 1, 1);
    Lattice lattice(3, 3, 3, blocks, threads, FluidData(1.0, 1.0), 0.5);
    LatticePoint* a = zeroed(27);
    lattice.load_data(a);
    delete[] a;
    lattice.insertModel(mesh("cube_angled.obj"));
    lattice.simulateCollision();
    lattice.preProcessModel();
    a = lattice.retrieve_data();
    const char* t = "CoordinatesTest.TestReflection";
    if (!a[13].reflections) {
        got(t, 223, NAN);
    } else {
        got(t, 223, a[13].reflections->reflection_weight[1 * 3 + 0]);
        got(t, 224, a[13].reflections->reflection_weight[1 * 3 + 1]);
        got(t, 225, a[13].reflections->reflection_weight[1 * 3 + 2]);
        got(t, 226, lattice.getReflectionDirection(&a[13], 3));
        got(t, 227, lattice.getReflectionDirection(&a[13], 4));
        got(t, 228, lattice.getReflectionDirection(&a[13], 5));
    }
    delete[] a;
}

// ------------------------------------------------------------------ ModelTest, GeometryTest
static void ModelTests()
{
    {
        Model m;
        m.importModel(mesh("triangle.obj"));
        got("ModelTest.importModel", 11, (double)m.getMesh().number_of_vertices());
    }
    {
        Model m;
        m.importModel(mesh("cube.obj"));
        got("ModelTest.isModelClosed", 20, m.isModelClosed());
        m.importModel(mesh("triangle.obj"));
        got("ModelTest.isModelClosed", 24, m.isModelClosed());
    }
    {
        Model m;
        m.importModel(mesh("cube.obj"));
        got("ModelTest.isPointInsideModel", 35, m.isPointInsideModel(Point_3(0.0, 0.0, 0.0)));
        got("ModelTest.isPointInsideModel", 39, m.isPointInsideModel(Point_3(2.0, 0.0, 0.0)));
    }
    {
        Model m;
        m.importModel(mesh("quad.obj"));
        got("ModelTest.checkErrorModel", 48, m.checkError());
    }
    {
        Model m;
        m.importModel(mesh("compat_cube.obj"));
        Point_3 r = m.reflectionVector(Point_3(0.5, 0.5, -1.0), Point_3(0.5, 0.5, 1.0));
        got("ModelTest.intersectionNormal", 63, r.x);
        got("ModelTest.intersectionNormal", 64, r.y);
        got("ModelTest.intersectionNormal", 65, r.z);
        r = m.reflectionVector(Point_3(0.5, 0.5, -1.0), Point_3(0.5, 0.5, -2.0));
        got("ModelTest.intersectionNormal", 73, r == Point_3(0.0, 0.0, 0.0));
    }
}

static void GeometryTests()
{
    Point_3 axis(cos(M_PI * 0.25), sin(M_PI * 0.25), 0.0), vector(1.0, 0.0, 0.0);
    Point_3 r = rotateVectorAroundAxis(axis, vector, 180.0 * (M_PI / 180.0));
    got("GeometryTest.TestQuaternionRoatation", 21, r.x);
    got("GeometryTest.TestQuaternionRoatation", 22, r.y);
    got("GeometryTest.TestQuaternionRoatation", 23, r.z);
    r = rotateVectorAroundAxis(axis, vector, 90.0 * (M_PI / 180.0));
    got("GeometryTest.TestQuaternionRoatation", 29, r.x);
    got("GeometryTest.TestQuaternionRoatation", 30, r.y);
    got("GeometryTest.TestQuaternionRoatation", 31, r.z);
}

int main(int argc, char** argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s <mesh dir> [--host-only]\n", argv[0]);
        return 2;
    }
    g_dir = argv[1];
    const bool host_only = argc > 2 && std::string(argv[2]) == "--host-only";
    ModelTests();
    GeometryTests();
    CompressionTest();
    TestDistributeVector();
    if (host_only) return 0;
    TestStreaming();
    TestCollision();
    TestFull();
    TestReflections(false);
    TestReflections(true);
    TestReflectionsDeviceData();
    TestFlowGeneration(false);
    TestFlowGeneration(true);
    TestCoordsMatch();
    TestCoordinatesWithModel();
    TestReflection();
    return 0;
}
