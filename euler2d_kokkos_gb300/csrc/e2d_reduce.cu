// e2d_reduce.cu -- FP64 reductions over a state: the conservation audit
// (interior sums of rho, E, mx, my), the L1 difference of two states and the
// radial density profile of the Sedov post-processing.  Deterministic: a fixed number of blocks, a fixed per-thread
// stride order and a fixed tree, so repeated calls give identical bits.
#include "e2d_internal.h"

#include <cmath>
#include <cstring>

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

// ------------------------------------------------------------ radial profile
// Ring index of array cell (i, j): src/ComputeRadialProfileFunctor.h:140-154,
// same operations in the same order (this file builds with --fmad=false).
__device__ __forceinline__ int ring_of(const ProfileGeom &g, int i, int j) {
  const double x = g.xmin + g.dx / 2 + (i - g.ghost) * g.dx;
  const double y = g.ymin + g.dy / 2 + (j - g.ghost) * g.dy;
  const double d = sqrt((x - g.cx) * (x - g.cx) + (y - g.cy) * (y - g.cy));
  return (int)(d / g.rmax * g.nbins);
}

// Largest |rho| over the counted cells (positive doubles order like their
// bit patterns) and a flag for non-finite values.
__global__ void __launch_bounds__(RT) k_profile_max(const ProfileGeom g, const double *__restrict__ rho,
                                                    unsigned long long *maxbits, unsigned int *flags) {
  unsigned long long m = 0ull;
  unsigned int bad = 0u;
  const long long n = (long long)g.isize * g.jsize;
  for (long long k = blockIdx.x * (long long)RT + threadIdx.x; k < n; k += (long long)gridDim.x * RT) {
    const int j = (int)(k / g.isize), i = (int)(k - (long long)j * g.isize);
    if (ring_of(g, i, j) >= g.nbins) continue;
    const double v = rho[k];
    if (isnan(v) || isinf(v)) {
      bad = 1u;
      continue;
    }
    const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(v));
    m = b > m ? b : m;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, m, off);
    m = o > m ? o : m;
  }
  bad = __reduce_or_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0) {
    if (m) atomicMax(maxbits, m);
    if (bad) atomicOr(flags, 1u);
  }
}

// Exact per-ring sums: each |rho| is scaled by 2^S (S from the maximum, so
// every scaled value is < 2^94), rounded to an integer -- exact for values
// within 2^42 of the maximum -- and split into three 32-bit limbs; the limbs
// and the counts are summed as 64-bit integers, so the result does not
// depend on the order of the additions.  SMEM: per-block partial sums in
// shared memory first (nbins <= kProfileSmemRings).
template <bool SMEM>
__global__ void __launch_bounds__(RT) k_profile_sums(const ProfileGeom g, const double *__restrict__ rho,
                                                     const unsigned long long *maxbits,
                                                     unsigned long long *__restrict__ acc) {
  extern __shared__ unsigned long long sacc[];  // [4][nbins]: count, limb0, limb1, limb2
  const int nb = g.nbins;
  unsigned long long *dst = acc;
  if (SMEM) {
    for (int k = threadIdx.x; k < 4 * nb; k += RT) sacc[k] = 0ull;
    __syncthreads();
    dst = sacc;
  }
  const double maxv = __longlong_as_double((long long)*maxbits);
  int e = 0;
  if (maxv > 0.0) frexp(maxv, &e);
  const int S = 94 - e;
  const long long n = (long long)g.isize * g.jsize;
  for (long long k = blockIdx.x * (long long)RT + threadIdx.x; k < n; k += (long long)gridDim.x * RT) {
    const int j = (int)(k / g.isize), i = (int)(k - (long long)j * g.isize);
    const int b = ring_of(g, i, j);
    if (b >= nb) continue;
    const double v = rho[k];
    const double x = rint(ldexp(fabs(v), S));          // integer-valued, < 2^94
    const double l2 = floor(ldexp(x, -64));
    const double r = x - ldexp(l2, 64);                // exact: x mod 2^64
    const double l1 = floor(ldexp(r, -32));
    const double l0 = r - ldexp(l1, 32);               // exact
    unsigned long long q[3] = {(unsigned long long)l0, (unsigned long long)l1, (unsigned long long)l2};
    if (v < 0.0)
      for (int t = 0; t < 3; ++t) q[t] = 0ull - q[t];  // two's complement: signed sums
    atomicAdd(&dst[b], 1ull);
    for (int t = 0; t < 3; ++t)
      if (q[t]) atomicAdd(&dst[(t + 1) * nb + b], q[t]);
  }
  if (SMEM) {
    __syncthreads();
    for (int k = threadIdx.x; k < 4 * nb; k += RT)
      if (sacc[k]) atomicAdd(&acc[k], sacc[k]);
  }
}

}  // namespace

cudaError_t launch_radial_profile(const ProfileGeom &g, const double *rho, unsigned long long *scratch,
                                  unsigned int *flags, cudaStream_t s) {
  // scratch: [0] max bits, [1 .. 4*nbins] count and limbs per ring
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * (1 + 4 * (size_t)g.nbins), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  k_profile_max<<<RBLOCKS, RT, 0, s>>>(g, rho, scratch, flags);
  if (g.nbins <= kProfileSmemRings) {
    const size_t smem = sizeof(unsigned long long) * 4 * (size_t)g.nbins;
    if (smem > 48 * 1024) {
      e = cudaFuncSetAttribute(k_profile_sums<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    k_profile_sums<true><<<RBLOCKS, RT, smem, s>>>(g, rho, scratch, scratch + 1);
  } else {
    k_profile_sums<false><<<RBLOCKS, RT, 0, s>>>(g, rho, scratch, scratch + 1);
  }
  return cudaGetLastError();
}

void finish_radial_profile(const ProfileGeom &g, const unsigned long long *host_scratch, double *profile,
                           long long *counts) {
  const int nb = g.nbins;
  const double maxv = [&] {
    double m;
    std::memcpy(&m, &host_scratch[0], sizeof m);
    return m;
  }();
  int e = 0;
  if (maxv > 0.0) std::frexp(maxv, &e);
  const int S = 94 - e;
  const unsigned long long *acc = host_scratch + 1;
  for (int b = 0; b < nb; ++b) {
    const long long cnt = (long long)acc[b];
    __int128 tot = (__int128)(long long)acc[3 * nb + b];
    tot = tot * ((__int128)1 << 32) + (__int128)(long long)acc[2 * nb + b];
    tot = tot * ((__int128)1 << 32) + (__int128)(long long)acc[nb + b];
    const double sum = std::ldexp((double)tot, -S);    // one rounding
    if (counts) counts[b] = cnt;
    profile[b] = sum / (double)cnt;                     // 0/0 = NaN for an empty ring, as in the reference
  }
}

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
