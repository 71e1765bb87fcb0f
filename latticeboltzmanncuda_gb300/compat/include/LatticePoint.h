// Compatibility header: the reference's state record and reflection table (LatticePoint.h:3-17),
// same layout (144 and 380 bytes), so that arrays of them pass through unchanged.
#pragma once

struct ReflectionValues
{
    int reflection_directions[14];   // 81 slots of 5-bit directions, 6 per int
    float reflection_weight[81];     // slot 3 * population + k, k < 3
};

struct LatticePoint
{
    int x, y, z;
    float particle_distribution[27];
    bool isReflected;
    bool isInternal;
    ReflectionValues* reflections = nullptr;    // host table of a reflecting cell (retrieve_data)
    ReflectionValues* d_reflections = nullptr;  // not used by this implementation (always null)
};

static_assert(sizeof(ReflectionValues) == 380, "ReflectionValues layout");
static_assert(sizeof(LatticePoint) == 144, "LatticePoint layout");
