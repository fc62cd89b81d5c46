// Minimal host-only stand-in for the Kokkos macro header.
//
// Test infrastructure only: it exists so that the reference solver's own
// headers (HydroBaseFunctor.h, HydroRunFunctors.h, HydroRun.h, HydroParams.cpp)
// compile unmodified on the CPU and can serve as the parity checker for the
// GPU path.  Nothing in the product links against it.
#pragma once

#define KOKKOS_VERSION_MAJOR 5
#define KOKKOS_VERSION_MINOR 1
#define KOKKOS_VERSION_PATCH 0
#define KOKKOS_ENABLE_CXX17 1
#define KOKKOS_ENABLE_SERIAL 1

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
