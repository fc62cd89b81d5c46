// Host-only stand-in for the Kokkos math wrappers the reference imports
// (real_type.h uses Kokkos::{exp,fmax,fmin,sqrt,fabs,fmod,isnan}).
// Each forwards to the C library, which is what Kokkos' host backends do.
#pragma once
#include <cmath>

namespace Kokkos
{
using std::exp;
using std::fabs;
using std::fmax;
using std::fmin;
using std::fmod;
using std::isnan;
using std::sqrt;
} // namespace Kokkos
