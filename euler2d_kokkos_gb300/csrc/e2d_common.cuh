// e2d_common.cuh -- device helpers shared by the FP64 and FP32 kernels.
#pragma once

#include "e2d_internal.h"

namespace e2d {

// Source cell of a ghost along one axis: the composition of the X-face pass
// (all rows) and the Y-face pass (all columns) of MakeBoundariesFunctor
// (src/HydroRunFunctors.h:1855-2024).  Reflect mirrors (2g-1-i) and flips
// the normal momentum, absorb copies the first interior cell, periodic
// wraps.  With n >= 2 the result is always an interior cell, so a ghost never
// reads another ghost and corners follow the X-then-Y fill order.
__device__ __forceinline__ int ghost_source(int i, int n, int bc_lo, int bc_hi, bool &flip) {
  flip = false;
  if (i < 2) {
    if (bc_lo == E2D_BC_REFLECT) {
      flip = true;
      return 3 - i;
    }
    if (bc_lo == E2D_BC_ABSORB) return 2;
    return n + i;
  }
  if (i >= n + 2) {
    if (bc_hi == E2D_BC_REFLECT) {
      flip = true;
      return 2 * n + 3 - i;
    }
    if (bc_hi == E2D_BC_ABSORB) return n + 1;
    return i - n;
  }
  return i;
}

__device__ __forceinline__ bool nonfinite64(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7ff) == 0x7ff;
}

}  // namespace e2d
