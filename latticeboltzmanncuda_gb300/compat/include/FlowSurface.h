// Compatibility header for FlowSurface.h of the reference (FlowSurface.h:9-46): an induced flow
// (populations added each flow pass) and the predicate of the cells that receive it.
#pragma once

#include "FlowCriterion.cuh"
#include "LatticePoint.h"

struct FlowData
{
    LatticePoint inducedFlow;
    bool (*pointCriterion)(int x, int y, int z) = nullptr;
    int val = 1;

    // criterion: address of a predicate pointer, e.g. &FlowCriterion::ptestPlaneCriteria
    FlowData(bool (**criterion)(int, int, int), LatticePoint flow) : inducedFlow(flow)
    {
        pointCriterion = criterion ? *criterion : nullptr;
    }

    void setCriterion(bool (**criterion)(int, int, int)) { pointCriterion = criterion ? *criterion : nullptr; }

    void setInducedFlow(LatticePoint flow) { inducedFlow = flow; }
};
