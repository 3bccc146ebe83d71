// Force-included before the reference headers when the reference's CPU
// driver is compiled as the oracle with g++ (no CUDA, no Eigen, C++14).
//
// TEST INFRASTRUCTURE ONLY.  It supplies what the reference headers assume
// from MSVC / nvcc but never include themselves:
//   * <cstdint> for uint8_t (gcurval/base/functors.inl.h:276),
//   * std::fabsl (gcurval/base/util.h:130; libstdc++ only has ::fabsl),
//   * an empty __constant__ qualifier (gcurval/base/constants.inl.h:10,97-98)
//     because USE_CUDA is not defined for the CPU build.
#pragma once

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <math.h>
#include <numeric>
#include <vector>

namespace std
{
using ::fabsl;
}

#ifndef __constant__
#define __constant__
#endif
