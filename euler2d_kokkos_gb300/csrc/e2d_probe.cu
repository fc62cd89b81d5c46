// e2d_probe.cu -- throughput of this GPU's FP64 operations, the denominator
// of the FP64-pipe roofline of the FP64 step (which GB300's FP64 pipe, not
// HBM, bounds).  Each thread runs 8 independent dependency chains of one
// operation so that the pipe, not latency, limits the rate; every SM runs
// 8 blocks of 256 threads.  Built with --fmad=false like the FP64 kernels, so
// division and square root are the same instruction sequences they run.
#include "e2d_internal.h"

#include <cuda_runtime.h>

namespace e2d {
namespace {

enum Op { OP_FMA = 0, OP_ADD, OP_MUL, OP_DIV, OP_SQRT, OP_MAX, OP_COUNT };
constexpr int kChains = 8;

template <int OP>
__global__ void __launch_bounds__(256) k_fp64_probe(double *out, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) x[k] = 1.0 + 1e-3 * k + 1e-9 * threadIdx.x;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) {
      if (OP == OP_FMA) x[k] = fma(x[k], a, b);  // fixed point b / (1 - a)
      if (OP == OP_ADD) x[k] = x[k] + b;         // b: far below an ulp of x
      if (OP == OP_MUL) x[k] = x[k] * a;         // a: 1 at run time
      if (OP == OP_DIV) x[k] = a / x[k];         // x alternates near 1 and a
      if (OP == OP_SQRT) x[k] = sqrt(x[k]);      // tends to 1
      if (OP == OP_MAX) x[k] = fmax(x[k], b);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += x[k];
  if (s == 12345.0) out[blockIdx.x] = s;  // keeps the chains live
}

template <int OP>
float time_op(double *out, int blocks, int iters, double a, double b, cudaStream_t st, cudaEvent_t e0,
              cudaEvent_t e1, cudaError_t *err) {
  k_fp64_probe<OP><<<blocks, 256, 0, st>>>(out, iters / 8, a, b);  // warm-up
  cudaEventRecord(e0, st);
  k_fp64_probe<OP><<<blocks, 256, 0, st>>>(out, iters, a, b);
  cudaEventRecord(e1, st);
  *err = cudaEventSynchronize(e1);
  if (*err == cudaSuccess) *err = cudaGetLastError();
  float ms = 0.f;
  if (*err == cudaSuccess) *err = cudaEventElapsedTime(&ms, e0, e1);
  return ms;
}

}  // namespace
}  // namespace e2d

using namespace e2d;

extern "C" int e2d_fp64_rates(double rates[6]) {
  if (!rates) return E2D_EINVAL;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
    return E2D_ECUDA;
  const int blocks = sms * 8;
  double *out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int status = E2D_OK;
  if (cudaMalloc(&out, sizeof(double) * blocks) != cudaSuccess) return E2D_ENOMEM;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    status = E2D_ECUDA;
  } else {
    // iterations per chain: ~10 ms per launch at the expected rates
    const int iters[OP_COUNT] = {2048, 2048, 2048, 256, 256, 4096};
    for (int op = 0; op < OP_COUNT && status == E2D_OK; ++op) {
      cudaError_t err = cudaSuccess;
      float ms = 0.f;
      switch (op) {
        case OP_FMA: ms = time_op<OP_FMA>(out, blocks, iters[op], 0.999, 1e-3, st, e0, e1, &err); break;
        case OP_ADD: ms = time_op<OP_ADD>(out, blocks, iters[op], 1.0, 1e-30, st, e0, e1, &err); break;
        case OP_MUL: ms = time_op<OP_MUL>(out, blocks, iters[op], 1.0, 0.0, st, e0, e1, &err); break;
        case OP_DIV: ms = time_op<OP_DIV>(out, blocks, iters[op], 1.0000001, 0.0, st, e0, e1, &err); break;
        case OP_SQRT: ms = time_op<OP_SQRT>(out, blocks, iters[op], 0.0, 0.0, st, e0, e1, &err); break;
        default: ms = time_op<OP_MAX>(out, blocks, iters[op], 0.0, 0.5, st, e0, e1, &err); break;
      }
      if (err != cudaSuccess || ms <= 0.f) {
        status = E2D_ECUDA;
        break;
      }
      rates[op] = (double)blocks * 256.0 * kChains * iters[op] / (ms * 1e-3) / 1e9;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  cudaFree(out);
  return status;
}
