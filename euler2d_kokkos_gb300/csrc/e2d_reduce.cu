// e2d_reduce.cu -- FP64 reductions over the interior of a state: the
// conservation audit (sums of rho, E, mx, my) and the L1 difference of two
// states.  Deterministic: a fixed number of blocks, a fixed per-thread
// stride order and a fixed tree, so repeated calls give identical bits.
#include "e2d_internal.h"

namespace e2d {
namespace {

constexpr int RT = 256;      // threads per block
constexpr int RBLOCKS = 608; // 4 x 152 SMs

__device__ __forceinline__ double block_sum(double x, double *sh) {
  const int tid = threadIdx.x;
  sh[tid] = x;
  __syncthreads();
  for (int s = RT / 2; s > 0; s >>= 1) {
    if (tid < s) sh[tid] += sh[tid + s];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// partial[b * nv + v] = sum over the cells visited by block b.
__global__ void __launch_bounds__(RT) k_sums(const KGeom g, const double *__restrict__ u,
                                             double *__restrict__ partial) {
  __shared__ double sh[RT];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const long long ncell = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)RT + threadIdx.x; k < ncell; k += (long long)RBLOCKS * RT) {
    const int j = (int)(k / g.nx), i = (int)(k - (long long)j * g.nx);
    const long long c = (i + 2) + (long long)g.isize * (j + 2);
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[v] += u[c + v * g.plane];
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const double s = block_sum(acc[v], sh);
    if (threadIdx.x == 0) partial[blockIdx.x * 4 + v] = s;
  }
}

__global__ void __launch_bounds__(RT) k_l1diff(const KGeom g, const double *__restrict__ a,
                                               const double *__restrict__ b, const int var,
                                               double *__restrict__ partial) {
  __shared__ double sh[RT];
  double da = 0.0, db = 0.0;
  const long long ncell = (long long)g.nx * g.ny;
  const double *pa = a + var * g.plane, *pb = b + var * g.plane;
  for (long long k = blockIdx.x * (long long)RT + threadIdx.x; k < ncell; k += (long long)RBLOCKS * RT) {
    const int j = (int)(k / g.nx), i = (int)(k - (long long)j * g.nx);
    const long long c = (i + 2) + (long long)g.isize * (j + 2);
    da += fabs(pa[c] - pb[c]);
    db += fabs(pb[c]);
  }
  const double s0 = block_sum(da, sh);
  const double s1 = block_sum(db, sh);
  if (threadIdx.x == 0) {
    partial[blockIdx.x * 2] = s0;
    partial[blockIdx.x * 2 + 1] = s1;
  }
}

// out[v] = sum over blocks of partial[b * nv + v], one block, fixed tree.
__global__ void __launch_bounds__(RT) k_finish(const double *__restrict__ partial, const int nv,
                                               double *__restrict__ out) {
  __shared__ double sh[RT];
  for (int v = 0; v < nv; ++v) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < RBLOCKS; b += RT) acc += partial[b * nv + v];
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) out[v] = s;
  }
}

}  // namespace

size_t reduce_partial_count(const KGeom &) { return (size_t)RBLOCKS * 4; }

cudaError_t launch_sums_f64(const KGeom &g, const double *u, double *partial, double *out4, cudaStream_t s) {
  k_sums<<<RBLOCKS, RT, 0, s>>>(g, u, partial);
  k_finish<<<1, RT, 0, s>>>(partial, 4, out4);
  return cudaGetLastError();
}

cudaError_t launch_l1diff_f64(const KGeom &g, const double *a, const double *b, int var,
                              double *partial, double *out2, cudaStream_t s) {
  k_l1diff<<<RBLOCKS, RT, 0, s>>>(g, a, b, var, partial);
  k_finish<<<1, RT, 0, s>>>(partial, 2, out2);
  return cudaGetLastError();
}

}  // namespace e2d
