// Compatibility header for Lattice.h of the reference (Lattice.h:1-106) on the library's C ABI
// (include/lbm_capi.h, mode LBM_D3Q27_REF).  Same classes, methods and argument meaning; the
// differences a caller can see:
//   * the populations live on the device as structure of arrays, not as pitched LatticePoint
//     records: getCudaDataPointer() returns a handle (ptr = the library context) that the
//     RunCudaFunctions launchers accept, not a device address of records;
//   * dim3 blocks/threads are accepted and ignored (the library picks its launch shapes);
//   * errors are printed as in the reference, and also available from lastError().
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <string>
#include <utility>
#include <vector>

#include "FlowSurface.h"
#include "Geometry.h"
#include "LatticePoint.h"

class Model;
struct lbm_ctx;

struct LatticeData
{
    cudaPitchedPtr latticePtr;
    dim3 latticeDimensions;

    LatticeData(cudaPitchedPtr ptr, dim3 dims) : latticePtr(ptr), latticeDimensions(dims) {}
    LatticeData() : latticePtr(cudaPitchedPtr()), latticeDimensions(dim3()) {}
};

struct FluidData
{
    float m_fluidDensity;
    float m_characteristicTimescale;

    FluidData(float fluidDensity, float characteristicTimescale)
        : m_fluidDensity(fluidDensity), m_characteristicTimescale(characteristicTimescale) {}
    FluidData() : m_fluidDensity(1.0), m_characteristicTimescale(1.0) {}
};

struct ReflectionData
{
    float x = 0.0;
    float y = 0.0;
    float z = 0.0;
};

class Lattice
{
public:
    Lattice(int x, int y, int z, dim3 blocks, dim3 threads, FluidData fluid, float spacing);
    ~Lattice();
    Lattice(const Lattice&) = delete;
    Lattice& operator=(const Lattice&) = delete;

    void load_data(LatticePoint* lattice_array);
    LatticePoint* retrieve_data();                  // new[] array owned by the caller, or nullptr
    ReflectionData* retrieve_reflection_data();     // the object given to setReflectionData, updated

    dim3 getDimensions() { return dim3(m_xResolution, m_yResolution, m_zResolution); }
    cudaPitchedPtr getCudaDataPointer();

    void simulateStreaming();
    void simulateCollision();
    void simulateReflections();
    void simulateFlow();

    void simulateLattice();                         // streaming then collision, as one fused step

    void insertModel(std::string filename);

    std::array<std::pair<float, int>, 27> distributeVector(Point_3 vector);

    void preProcessModel();

    void setFlowData(FlowData* flowData);

    void setReflectionData(ReflectionData* reflection);

    void setReflectionDirection(LatticePoint* point, const int index, const unsigned int value);
    int getReflectionDirection(LatticePoint* point, const int index);

    // ---- additions (no counterpart in the reference)
    // nsteps fused steps in the CLI order: streaming, reflections, collision, flow
    void simulateSteps(int nsteps);
    // the same, returning the accumulated reflection force after every step (setReflectionData first)
    std::vector<ReflectionData> simulateStepsWithForce(int nsteps);
    lbm_ctx* context() { return m_ctx; }
    const std::string& lastError() const { return m_error; }

private:
    bool ok(int status, const char* where);
    void refreshFlags(std::vector<unsigned char>& flags);

    lbm_ctx* m_ctx = nullptr;
    FluidData m_fluid;
    FlowData* m_flowData = nullptr;
    ReflectionData* m_reflectionData = nullptr;
    Model* m_simModel = nullptr;

    unsigned short m_xResolution;
    unsigned short m_yResolution;
    unsigned short m_zResolution;
    float m_latticeSpacing;
    dim3 m_threads;
    dim3 m_blocks;

    std::vector<ReflectionValues> m_reflections;    // host tables, in the order of m_reflectionCells
    std::vector<int> m_reflectionCells;
    std::string m_error;
};
