// Compatibility header for SimCalcFuncs.cuh of the reference (SimCalcFuncs.cuh:13-25): the single
// passes on a lattice named by LatticeData (built from Lattice::getCudaDataPointer()).  blocks and
// threads are ignored.  templattice is not needed (the library keeps its own second buffer) and may
// be any LatticeData.  The reference's kernels themselves (CudaFunctions::*) operate on pitched
// LatticePoint records and are not part of this interface.
#pragma once

#include <cuda_runtime.h>

#include "FlowSurface.h"
#include "Lattice.h"

namespace RunCudaFunctions
{
    void run_calculate_streaming(dim3 blocks, dim3 threads, LatticeData lattice, LatticeData templattice);

    void run_calculate_collision(dim3 blocks, dim3 threads, LatticeData lattice, float timescale);

    void run_calculate_reflections(dim3 blocks, dim3 threads, LatticeData lattice, LatticeData templattice);

    // reflections with the force added to *reflection (a host object here; a device pointer in the reference)
    void run_calculate_reflections_data(dim3 blocks, dim3 threads, LatticeData lattice, LatticeData templattice,
                                        ReflectionData* reflection);

    // coordinates are implicit in the library's layout: validates the lattice, nothing else
    void run_prime_points(dim3 blocks, dim3 threads, LatticeData lattice);

    void run_generate_flow(dim3 blocks, dim3 threads, LatticeData lattice, FlowData* flowData);
}
