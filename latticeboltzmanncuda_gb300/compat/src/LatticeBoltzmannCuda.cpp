// The reference's command line (LatticeBoltzmannCuda.cpp:11-96) on the compatibility layer:
//
//   LatticeBoltzmannCuda <model.obj> <threads x y z> <blocks x y z> <density> <timescale> <spacing> <steps>
//
// Same arguments and output: a lattice of threads * blocks cells per axis, every population 0.001
// (population 6: 0.002), the model's cells marked and their reflection tables built, the induced
// flow on the plane x = 0, and before every step the accumulated reflection force printed as
// "x y z".  The steps run fused (streaming, reflections, collision, flow in one pass plus the
// reflection gather) in chunks, with the force of every step recorded on the device and printed
// after each chunk, instead of one device-to-host copy and synchronisation per step.
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <vector>

#include "FlowCriterion.cuh"
#include "FlowSurface.h"
#include "Lattice.h"
#include "LatticePoint.h"

int main(int argc, char* argv[])
{
    if (argc < 12) {
        std::fprintf(stderr,
                     "usage: %s <model.obj> <threads x y z> <blocks x y z> <density> <timescale> <spacing> <steps>\n",
                     argc > 0 ? argv[0] : "LatticeBoltzmannCuda");
        return -1;
    }

    dim3 threads(atoi(argv[2]), atoi(argv[3]), atoi(argv[4]));
    dim3 blocks(atoi(argv[5]), atoi(argv[6]), atoi(argv[7]));
    FluidData fluid(atof(argv[8]), atof(argv[9]));
    const int steps = atoi(argv[11]);

    Lattice userLattice(threads.x * blocks.x, threads.y * blocks.y, threads.z * blocks.z, blocks, threads, fluid,
                        atof(argv[10]));
    if (!userLattice.context()) return 1;

    LatticePoint flowRef;
    for (int i = 0; i < 27; ++i) flowRef.particle_distribution[i] = 0.001f;
    flowRef.particle_distribution[6] = 0.002f;

    LatticePoint* data = userLattice.retrieve_data();
    if (!data) return 1;
    const size_t cells = (size_t)threads.x * blocks.x * threads.y * blocks.y * threads.z * blocks.z;
    for (size_t c = 0; c < cells; ++c)
        for (int i = 0; i < 27; ++i) data[c].particle_distribution[i] = flowRef.particle_distribution[i];
    userLattice.load_data(data);
    delete[] data;

    userLattice.insertModel(argv[1]);
    userLattice.preProcessModel();

    FlowData inducedFlow(&FlowCriterion::ptestPlaneCriteria, flowRef);
    userLattice.setFlowData(&inducedFlow);

    ReflectionData reflection;
    userLattice.setReflectionData(&reflection);

    // line k is the force after k steps, k = 0 .. steps - 1
    int printed = 0;
    if (steps > 0) {
        std::cout << reflection.x << " " << reflection.y << " " << reflection.z << "\n";
        ++printed;
    }
    const int chunk = 4096;
    for (int done = 0; done < steps;) {
        const int n = std::min(chunk, steps - done);
        const std::vector<ReflectionData> series = userLattice.simulateStepsWithForce(n);
        if ((int)series.size() != n) return 1;
        for (const ReflectionData& r : series) {
            if (printed >= steps) break;
            std::cout << r.x << " " << r.y << " " << r.z << "\n";
            ++printed;
        }
        std::cout.flush();
        done += n;
    }
    return 0;
}
