// Force-included when compiling the reference's host sources for the oracle tests: the
// reference calls unqualified isnan (thirdparty/RadeonRays/split_bvh.cpp:79,104), which
// MSVC provides globally and libstdc++ only through <cmath> in namespace std.
#pragma once
#include <cmath>
using std::isnan;
