// Compatibility header for FlowCriterion.cuh of the reference (FlowCriterion.cu:3-17).
//
// The reference selects the flow-source cells with a __device__ predicate reached through a
// __device__ function pointer.  Here the predicates are host functions: Lattice::setFlowData
// evaluates the FlowData's predicate once per cell on the host and hands the resulting mask to the
// library, so any host predicate with this signature works.
#pragma once

namespace FlowCriterion
{
    bool testCriteria(int x, int y, int z);       // the single cell (1, 1, 1)
    bool testPlaneCriteria(int x, int y, int z);  // the plane x = 0

    extern bool (*ptestCriteria)(int, int, int);
    extern bool (*ptestPlaneCriteria)(int, int, int);
}
