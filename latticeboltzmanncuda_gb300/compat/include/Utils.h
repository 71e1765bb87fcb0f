// Compatibility header for Utils.h of the reference (Utils.cpp:9-37).
#pragma once

namespace Utils
{
    // packs num values of bitLength bits into one word, 5 bits apart, first value highest
    unsigned int compressInts(int* array, const int num, const int bitLength);
}
