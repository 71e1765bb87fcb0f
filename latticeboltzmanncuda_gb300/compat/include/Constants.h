// Compatibility header for Constants.h of the reference (Constants.cpp:3-8).
#ifndef CONSTANTS_H
#define CONSTANTS_H

namespace CONSTANTS
{
    extern const float GEOMETRIC_TOLERANCE;
    extern const int DIRECTIONS[27][3];
    extern const int INVERSE_DIRECTIONS[27];
}

#endif
