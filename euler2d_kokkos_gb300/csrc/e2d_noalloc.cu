// e2d_noalloc.cu -- one FP64 time step on caller-owned device buffers that
// allocates no memory.
//
// Some callers cannot let a library call cudaMalloc: hosts that hand out all
// device memory from their own fixed pool and forbid hidden allocations,
// latency-critical loops where cudaMalloc's implicit device synchronisation
// is not acceptable, and code that has no handle to keep (a plain C call per
// step).  For them e2d_godunov_unsplit_noalloc runs the same two kernels as
// e2d_godunov_unsplit, with their scratch -- the primitives array and the
// device clock -- in a file-scope __device__ array of fixed size instead of
// handle-owned allocations.  Every GPU that loads the library holds that
// array (E2D_NOALLOC_MAX_CELLS * 32 B plus a few hundred bytes) until the
// process exits.
#include <mutex>

#include "e2d_internal.h"

namespace e2d {
namespace {

constexpr long long kMaxCells = E2D_NOALLOC_MAX_CELLS;
constexpr size_t kClockDoubles = (sizeof(DevClock) + sizeof(double) - 1) / sizeof(double);

// Scratch shared by every call on a device: primitives of up to kMaxCells
// cells (4 doubles each), then the device clock.  Host code must not use
// this name as an address: it is the host-side stand-in of the symbol.
static __device__ __align__(256) double g_noalloc_scratch[4 * kMaxCells + kClockDoubles];

constexpr int kMaxDevices = 64;
double *g_scratch_ptr[kMaxDevices] = {};  // device address of the scratch, per device
std::mutex g_setup_mutex;

// Once per device, with that device current: the device address of the
// scratch symbol and the kernels' shared-memory limit.  Both are kept for the
// life of the process; after a cudaDeviceReset the cached address would be
// stale, so calls after a reset are not supported (include/e2d.h says so).
int setup_device(int dev, double **out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    double *ptr = nullptr;
    if (cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return E2D_ECUDA;
    if (configure_f64_kernels() != cudaSuccess) return E2D_ECUDA;
    g_scratch_ptr[dev] = ptr;
  }
  *out = g_scratch_ptr[dev];
  return E2D_OK;
}

}  // namespace
}  // namespace e2d

using namespace e2d;

extern "C" int e2d_godunov_unsplit_noalloc(const e2d_params *pin, double *u_in, double *u_out,
                                           double dt, void *stream) {
  if (!pin || !u_in || !u_out || u_in == u_out) return E2D_EINVAL;
  e2d_params p = *pin;
  int rc = params_init(&p, nullptr);
  if (rc != E2D_OK) return rc;
  if (p.precision != E2D_PRECISION_FP64) return E2D_EINVAL;
  // grids beyond the fixed scratch are refused, never truncated
  if ((long long)p.isize * p.jsize > kMaxCells) return E2D_EINVAL;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return E2D_ECUDA;
  if (dev < 0 || dev >= kMaxDevices) return E2D_EINVAL;
  double *scratch = nullptr;
  rc = setup_device(dev, &scratch);
  if (rc != E2D_OK) return rc;
  double *q = scratch;
  DevClock *clk = reinterpret_cast<DevClock *>(scratch + 4 * kMaxCells);
  KParams64 kp;
  make_kparams(p, &kp);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the primitives kernel writes every cell of q before the flux kernel reads
  // it, and neither kernel reads the clock in this mode: nothing left over
  // from an earlier call is used
  if (launch_fill_f64(kp, u_in, u_out, q, clk, FILL_WRITE_Q | FILL_GHOSTS_IN | FILL_GHOSTS_OUT, s) != cudaSuccess)
    return E2D_ECUDA;
  if (launch_flux_update_f64(kp, p.riemannSolverType, q, u_in, u_out, clk, 0, dt, nullptr, s) != cudaSuccess)
    return E2D_ECUDA;
  return E2D_OK;
}
