// e2d_capi.cu -- the C ABI of include/e2d.h: simulation handles, device
// buffers, the HydroRun method mirrors and the graph-replayed time loop, for
// both arithmetic modes (FP64 bit-identical, FP32 compensated).
#include "e2d_internal.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

using namespace e2d;

struct e2d_sim {
  e2d_params p{};
  KParams64 kp{};
  KParams32 kp32{};
  int fp32 = 0;                       // precision == E2D_PRECISION_FP32C
  int device = 0;
  cudaStream_t stream = nullptr;
  double *U[2] = {nullptr, nullptr};  // FP64: U and U2 of the reference
  double *Q[2] = {nullptr, nullptr};  // FP64: primitives of U and of U2 (the fused step's ping-pong;
                                      // Q[0] is the two-launch step's scratch)
  CUtensorMap QTM[2];                 // FP64: TMA maps of Q[0], Q[1] (fused step's tile staging)
  int q_tma = 0;                      // FP64: both maps encoded (isize even)
  int f64_split = 0;                  // FP64 device loop as two launches per step (E2D_F64_SPLIT=1)
  int impl = 0;                       // FP64: implementationVersion (1, 2: the debug orchestrations)
  // FP64 fused step: the parity whose primitives (Q[par], interior) and CFL
  // maximum (q_acc) on the device are those of U[par] as the last device-loop
  // call left them, so the next call needs no prologue; -1 once anything may
  // have changed a state
  int q_ready = -1;
  unsigned long long q_acc = 0ull;
  double *impl_scratch = nullptr;     // FP64, implementation 1: stored slopes and fluxes
  float *W[2] = {nullptr, nullptr};   // FP32C: compensated U and U2 (8 float planes)
  CUtensorMap TM[2];                  // FP32C: TMA maps of W[0], W[1] (row staging)
  double *stage = nullptr;            // FP32C: FP64 staging array (set/get/init)
  double *partial = nullptr;          // reduction partials
  double *red_out = nullptr;          // reduction results (device)
  DevClock *clk = nullptr;            // device loop state
  DevClock *clk_host = nullptr;       // pinned mirror
  double *dt_trace = nullptr;         // device dt trace
  int dt_trace_cap = 0;
  std::string err;
  // cached graphs: key = (steps << 1) | parity of the first input buffer
  std::map<int, cudaGraphExec_t> graphs;
  // per-kernel profiling
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::map<std::string, double> k_ms;
  std::map<std::string, long> k_count;
  std::vector<std::string> k_names;
};

namespace {

constexpr int kGraphSteps = 8;  // steps captured per cached graph

int set_err(e2d_sim *s, int status, const std::string &msg) {
  if (s) s->err = msg;
  return status;
}

int cuda_fail(e2d_sim *s, cudaError_t e, const char *what) {
  if (e == cudaErrorMemoryAllocation)
    return set_err(s, E2D_ENOMEM, std::string(what) + ": " + cudaGetErrorString(e));
  return set_err(s, E2D_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define E2D_CK(sim, call, what)                               \
  do {                                                        \
    cudaError_t e__ = (call);                                 \
    if (e__ != cudaSuccess) return cuda_fail(sim, e__, what); \
  } while (0)

}  // namespace

void e2d::make_kparams(const e2d_params &p, KParams64 *kp) {
  kp->g.nx = p.nx;
  kp->g.ny = p.ny;
  kp->g.isize = p.isize;
  kp->g.jsize = p.jsize;
  kp->g.plane = (long long)p.isize * p.jsize;
  kp->g.bc_xmin = p.boundary_type_xmin;
  kp->g.bc_xmax = p.boundary_type_xmax;
  kp->g.bc_ymin = p.boundary_type_ymin;
  kp->g.bc_ymax = p.boundary_type_ymax;
  kp->ph.gamma0 = p.gamma0;
  kp->ph.gamma6 = p.gamma6;
  kp->ph.cfl = p.cfl;
  kp->ph.slope_type = p.slope_type;
  kp->ph.smallr = p.smallr;
  kp->ph.smallc = p.smallc;
  kp->ph.smallp = p.smallp;
  kp->ph.smallpp = p.smallpp;
  kp->ph.gm1 = p.gamma0 - 1.0;
  kp->ph.entho = 1.0 / (p.gamma0 - 1.0);
  kp->ph.smallc2 = p.smallc * p.smallc;
  kp->ph.dx = p.dx;
  kp->ph.dy = p.dy;
  auto inv_pow2 = [](double d) {
    int e = 0;
    const double m = std::frexp(d, &e);  // d = m * 2^e, m in [0.5, 1)
    return (m == 0.5 && 1 - e >= -1022 && 1 - e <= 1023) ? std::ldexp(1.0, 1 - e) : 0.0;
  };
  kp->ph.inv_dx_pow2 = inv_pow2(p.dx);
  kp->ph.inv_dy_pow2 = inv_pow2(p.dy);
  kp->ph.inv_dx = 1.0 / p.dx;
  kp->ph.inv_dy = 1.0 / p.dy;
  kp->fast = p.precision == E2D_PRECISION_FP64_FAST ? 1 : 0;
  kp->tile = -1;
  if (const char *v = std::getenv("E2D_F64_TILE")) kp->tile = std::atoi(v);
  const char *wt = std::getenv("E2D_TEST_WAIT_TIMEOUT");
  kp->wait_test = (wt && std::atoi(wt) != 0) ? 1 : 0;
}

namespace {

size_t cells(const e2d_sim *s) { return (size_t)s->p.isize * s->p.jsize; }

// LayoutRight (OpenMP backend) <-> LayoutLeft (CUDA backend) on the host.
void right_to_left(const e2d_params &p, const double *src, double *dst) {
  const size_t plane = (size_t)p.isize * p.jsize;
  for (int i = 0; i < p.isize; ++i)
    for (int j = 0; j < p.jsize; ++j)
      for (int v = 0; v < 4; ++v) dst[i + (size_t)p.isize * j + plane * v] = src[((size_t)i * p.jsize + j) * 4 + v];
}
void left_to_right(const e2d_params &p, const double *src, double *dst) {
  const size_t plane = (size_t)p.isize * p.jsize;
  for (int i = 0; i < p.isize; ++i)
    for (int j = 0; j < p.jsize; ++j)
      for (int v = 0; v < 4; ++v) dst[((size_t)i * p.jsize + j) * 4 + v] = src[i + (size_t)p.isize * j + plane * v];
}

const char *riemann_name(int r) {
  return r == E2D_RIEMANN_HLLC ? "hllc" : r == E2D_RIEMANN_HLL ? "hll" : "approx";
}

// Kernels of one step of the device time loop, input buffer `par`.
cudaError_t enqueue_step(e2d_sim *s, int par) {
  if (s->fp32)
    return launch_f32c_step(s->kp32, s->p.riemannSolverType, s->W[par], s->W[par ^ 1], s->TM[par], s->clk, 1,
                            0.0, s->stream);
  double *in = s->U[par], *out = s->U[par ^ 1];
  if (s->impl != 0) {
    const int m = FILL_WRITE_Q | FILL_GHOSTS_IN | FILL_COPY_OUT | FILL_DT | FILL_DEVICE_CLOCK;
    cudaError_t e = launch_fill_f64(s->kp, in, out, s->Q[0], s->clk, m, s->stream);
    if (e != cudaSuccess) return e;
    return launch_impl12_f64(s->kp, s->impl, s->p.riemannSolverType, s->Q[0], out, s->impl_scratch, s->clk, 1,
                             0.0, s->dt_trace, s->stream);
  }
  if (!s->f64_split)
    return launch_step_f64(s->kp, s->p.riemannSolverType, s->QTM[par], s->q_tma, s->Q[par], s->Q[par ^ 1], in,
                           out, s->clk, s->dt_trace, s->stream);
  const int mode = FILL_WRITE_Q | FILL_GHOSTS_IN | FILL_GHOSTS_OUT | FILL_DT | FILL_DEVICE_CLOCK;
  cudaError_t e = launch_fill_f64(s->kp, in, out, s->Q[0], s->clk, mode, s->stream);
  if (e != cudaSuccess) return e;
  return launch_flux_update_f64(s->kp, s->p.riemannSolverType, s->Q[0], in, out, s->clk, 1, 0.0,
                                s->dt_trace, s->stream);
}

// Before the fused FP64 steps of a device-loop call: the primitives of the
// input state and its CFL maximum, which the first step reads.
cudaError_t enqueue_prologue(e2d_sim *s, int par, int nstep) {
  if (s->fp32 || s->f64_split || s->impl != 0) return cudaSuccess;
  return launch_fill_f64(s->kp, s->U[par], nullptr, s->Q[par], s->clk, FILL_WRITE_Q | FILL_DT, s->stream, nstep & 1);
}

cudaEvent_t pool_event(e2d_sim *s, size_t k) {
  while (s->ev_pool.size() <= k) {
    cudaEvent_t ev;
    if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
    s->ev_pool.push_back(ev);
  }
  return s->ev_pool[k];
}

int get_graph(e2d_sim *s, int steps, int par, cudaGraphExec_t *out) {
  const int key = (steps << 1) | par;
  auto it = s->graphs.find(key);
  if (it != s->graphs.end()) {
    *out = it->second;
    return E2D_OK;
  }
  cudaGraph_t graph;
  E2D_CK(s, cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "capture begin");
  cudaError_t le = cudaSuccess;
  for (int k = 0; k < steps && le == cudaSuccess; ++k) le = enqueue_step(s, (par + k) & 1);
  cudaError_t ee = cudaStreamEndCapture(s->stream, &graph);
  if (le != cudaSuccess) return cuda_fail(s, le, "capture step");
  if (ee != cudaSuccess) return cuda_fail(s, ee, "capture end");
  cudaGraphExec_t exec;
  cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) return cuda_fail(s, ie, "graph instantiate");
  s->graphs[key] = exec;
  *out = exec;
  return E2D_OK;
}

int ensure_trace(e2d_sim *s, int n) {
  if (n <= s->dt_trace_cap) return E2D_OK;
  if (s->dt_trace) cudaFree(s->dt_trace);
  s->dt_trace = nullptr;
  s->dt_trace_cap = 0;
  // the trace pointer is baked into captured graphs: drop them
  for (auto &kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
  const int cap = n < 1024 ? 1024 : n;
  E2D_CK(s, cudaMalloc(&s->dt_trace, sizeof(double) * cap), "dt trace alloc");
  s->dt_trace_cap = cap;
  return E2D_OK;
}

// FP64 view of state `which` on the device: the state itself (FP64) or its
// hi + lo conversion into the staging array (FP32C).
int fp64_view(e2d_sim *s, int which, double **out) {
  if (!s->fp32) {
    *out = s->U[which];
    return E2D_OK;
  }
  E2D_CK(s, launch_f32c_to_f64(s->kp32, s->W[which], s->stage, s->stream), "fp32c to fp64");
  *out = s->stage;
  return E2D_OK;
}

void record_kernel(e2d_sim *s, const std::string &name, float ms) {
  if (!s->k_count.count(name)) s->k_names.push_back(name);
  s->k_ms[name] += ms;
  s->k_count[name] += 1;
}

}  // namespace

extern "C" {

int e2d_abi_version(void) { return E2D_ABI_VERSION; }

const char *e2d_status_string(int status) {
  switch (status) {
    case E2D_OK: return "ok";
    case E2D_EINVAL: return "invalid argument";
    case E2D_ENOMEM: return "out of memory";
    case E2D_ENUMERIC: return "numerical failure (NaN/Inf state or non-positive dt)";
    case E2D_ETIMEOUT: return "device wait timed out";
    case E2D_ECUDA: return "CUDA error";
    case E2D_EIO: return "cannot read or write a file";
    default: return "unknown status";
  }
}

int e2d_params_defaults(e2d_params *p) {
  if (!p) return E2D_EINVAL;
  params_defaults(p);
  return E2D_OK;
}

int e2d_params_from_ini(const char *path, e2d_params *p) {
  if (!path || !p) return E2D_EINVAL;
  IniMap m;
  const int rc = m.parse(path);
  if (rc < 0) return E2D_EIO;
  // like INIReader, a syntax error on some line still yields the keys parsed
  return params_from_ini(m, p, nullptr);
}

int e2d_params_init(e2d_params *p) {
  if (!p) return E2D_EINVAL;
  return params_init(p, nullptr);
}

int e2d_ini_get_string(const char *path, const char *section, const char *name, const char *dflt,
                       char *buf, size_t buflen) {
  if (!path || !section || !name || !buf || buflen == 0) return E2D_EINVAL;
  IniMap m;
  if (m.parse(path) < 0) return E2D_EIO;
  const std::string v = m.get_string(section, name, dflt ? dflt : "");
  const size_t n = v.size() < buflen - 1 ? v.size() : buflen - 1;
  std::memcpy(buf, v.data(), n);
  buf[n] = '\0';
  return E2D_OK;
}

int e2d_create(const e2d_params *pin, e2d_sim **out) {
  if (!pin || !out) return E2D_EINVAL;
  *out = nullptr;
  e2d_params p = *pin;
  std::string msg;
  int rc = params_init(&p, &msg);
  if (rc != E2D_OK) return rc;
  e2d_sim *s = new (std::nothrow) e2d_sim();
  if (!s) return E2D_ENOMEM;
  s->p = p;
  s->fp32 = (p.precision == E2D_PRECISION_FP32C) ? 1 : 0;
  make_kparams(p, &s->kp);
  make_kparams32(p, &s->kp32);
  if (const char *v = std::getenv("E2D_F32C_VARIANT")) s->kp32.variant = std::atoi(v);
  // strip heights are whole 16-row CFL fold units
  if (const char *v = std::getenv("E2D_F32C_STRIP_H"))
    if (std::atoi(v) > 0 && std::atoi(v) <= 512) s->kp32.strip_h = (std::atoi(v) + 15) / 16 * 16;
  auto fail = [&](int status) {
    e2d_destroy(s);
    return status;
  };
  if (cudaGetDevice(&s->device) != cudaSuccess) return fail(E2D_ECUDA);
  if (configure_f64_kernels() != cudaSuccess || configure_f32c_kernels() != cudaSuccess) return fail(E2D_ECUDA);
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(E2D_ECUDA);
  const size_t n = cells(s);
  if (s->fp32) {
    const size_t wn = (size_t)8 * s->kp32.wplane;
    for (int k = 0; k < 2; ++k) {
      if (cudaMalloc(&s->W[k], sizeof(float) * wn) != cudaSuccess) return fail(E2D_ENOMEM);
      if (cudaMemsetAsync(s->W[k], 0, sizeof(float) * wn, s->stream) != cudaSuccess) return fail(E2D_ECUDA);
      if (!encode_f32c_map(&s->TM[k], s->W[k], s->kp32)) return fail(E2D_ECUDA);
    }
    if (cudaMalloc(&s->stage, sizeof(double) * 4 * n) != cudaSuccess) return fail(E2D_ENOMEM);
  } else {
    for (int k = 0; k < 2; ++k) {
      if (cudaMalloc(&s->U[k], sizeof(double) * 4 * n) != cudaSuccess) return fail(E2D_ENOMEM);
      if (cudaMemsetAsync(s->U[k], 0, sizeof(double) * 4 * n, s->stream) != cudaSuccess) return fail(E2D_ECUDA);
    }
    for (int k = 0; k < 2; ++k) {
      if (cudaMalloc(&s->Q[k], sizeof(double) * 4 * n) != cudaSuccess) return fail(E2D_ENOMEM);
      if (cudaMemsetAsync(s->Q[k], 0, sizeof(double) * 4 * n, s->stream) != cudaSuccess) return fail(E2D_ECUDA);
    }
    s->q_tma = encode_q_map(&s->QTM[0], s->Q[0], s->kp) && encode_q_map(&s->QTM[1], s->Q[1], s->kp);
    if (!s->q_tma) std::memset(s->QTM, 0, sizeof(s->QTM));
    if (const char *v = std::getenv("E2D_F64_SPLIT")) s->f64_split = std::atoi(v) != 0;
    s->impl = (p.implementationVersion == 1 || p.implementationVersion == 2) ? p.implementationVersion : 0;
    if (s->kp.fast) {
      // the fast forms exist in the fused step of implementation 0 only
      if (s->impl != 0) return fail(E2D_EINVAL);
      s->f64_split = 0;
    }
    if (const size_t k = impl12_scratch_doubles(s->kp, s->impl))
      if (cudaMalloc(&s->impl_scratch, sizeof(double) * k) != cudaSuccess) return fail(E2D_ENOMEM);
  }
  if (cudaMalloc(&s->partial, sizeof(double) * reduce_partial_count(s->kp.g)) != cudaSuccess) return fail(E2D_ENOMEM);
  if (cudaMalloc(&s->red_out, sizeof(double) * 8) != cudaSuccess) return fail(E2D_ENOMEM);
  if (cudaMalloc(&s->clk, sizeof(DevClock)) != cudaSuccess) return fail(E2D_ENOMEM);
  if (cudaMallocHost(&s->clk_host, sizeof(DevClock)) != cudaSuccess) return fail(E2D_ENOMEM);
  std::memset(s->clk_host, 0, sizeof(DevClock));
  if (cudaMemsetAsync(s->clk, 0, sizeof(DevClock), s->stream) != cudaSuccess) return fail(E2D_ECUDA);
  if (ensure_trace(s, 1024) != E2D_OK) return fail(E2D_ENOMEM);
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return fail(E2D_ECUDA);
  *out = s;
  return E2D_OK;
}

int e2d_destroy(e2d_sim *s) {
  if (!s) return E2D_EINVAL;
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (auto &kv : s->graphs) cudaGraphExecDestroy(kv.second);
  for (auto ev : s->ev_pool) cudaEventDestroy(ev);
  for (int k = 0; k < 2; ++k) {
    if (s->U[k]) cudaFree(s->U[k]);
    if (s->W[k]) cudaFree(s->W[k]);
  }
  for (int k = 0; k < 2; ++k)
    if (s->Q[k]) cudaFree(s->Q[k]);
  if (s->impl_scratch) cudaFree(s->impl_scratch);
  if (s->stage) cudaFree(s->stage);
  if (s->partial) cudaFree(s->partial);
  if (s->red_out) cudaFree(s->red_out);
  if (s->clk) cudaFree(s->clk);
  if (s->clk_host) cudaFreeHost(s->clk_host);
  if (s->dt_trace) cudaFree(s->dt_trace);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return E2D_OK;
}

const char *e2d_last_error(const e2d_sim *s) { return s ? s->err.c_str() : "null handle"; }

int e2d_get_params(const e2d_sim *s, e2d_params *p) {
  if (!s || !p) return E2D_EINVAL;
  *p = s->p;
  return E2D_OK;
}

int e2d_get_stream(e2d_sim *s, void **stream) {
  if (!s || !stream) return E2D_EINVAL;
  *stream = (void *)s->stream;
  return E2D_OK;
}

int e2d_device_state(e2d_sim *s, int which, double **dptr) {
  if (!s || !dptr || (which != 0 && which != 1)) return E2D_EINVAL;
  s->q_ready = -1;  // the caller may write through the pointer
  int rc = fp64_view(s, which, dptr);
  if (rc != E2D_OK) return rc;
  if (s->fp32) E2D_CK(s, cudaStreamSynchronize(s->stream), "device_state sync");
  return E2D_OK;
}

int e2d_init_problem(e2d_sim *s) {
  if (!s) return E2D_EINVAL;
  s->q_ready = -1;
  if (s->fp32) {
    E2D_CK(s, launch_init_f64(s->kp, s->p, s->stage, s->stream), "init problem");
    E2D_CK(s, launch_f32c_from_f64(s->kp32, s->stage, s->W[0], s->stream), "init convert");
    E2D_CK(s, cudaMemcpyAsync(s->W[1], s->W[0], sizeof(float) * 8 * s->kp32.wplane, cudaMemcpyDeviceToDevice, s->stream), "init copy");
  } else {
    E2D_CK(s, launch_init_f64(s->kp, s->p, s->U[0], s->stream), "init problem");
    E2D_CK(s, cudaMemcpyAsync(s->U[1], s->U[0], sizeof(double) * 4 * cells(s), cudaMemcpyDeviceToDevice, s->stream), "init copy");
  }
  E2D_CK(s, cudaStreamSynchronize(s->stream), "init sync");
  return E2D_OK;
}

int e2d_set_state(e2d_sim *s, int which, const double *host, int layout) {
  if (!s || !host || (which != 0 && which != 1)) return set_err(s, E2D_EINVAL, "bad set_state args");
  if (layout != E2D_LAYOUT_LEFT && layout != E2D_LAYOUT_RIGHT) return set_err(s, E2D_EINVAL, "bad layout");
  s->q_ready = -1;
  const size_t n = 4 * cells(s);
  std::vector<double> tmp;
  const double *src = host;
  if (layout == E2D_LAYOUT_RIGHT) {
    tmp.resize(n);
    right_to_left(s->p, host, tmp.data());
    src = tmp.data();
  }
  double *dst = s->fp32 ? s->stage : s->U[which];
  E2D_CK(s, cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, s->stream), "set_state copy");
  if (s->fp32) E2D_CK(s, launch_f32c_from_f64(s->kp32, s->stage, s->W[which], s->stream), "set_state convert");
  E2D_CK(s, cudaStreamSynchronize(s->stream), "set_state sync");
  return E2D_OK;
}

int e2d_get_state(e2d_sim *s, int which, double *host, int layout) {
  if (!s || !host || (which != 0 && which != 1)) return set_err(s, E2D_EINVAL, "bad get_state args");
  if (layout != E2D_LAYOUT_LEFT && layout != E2D_LAYOUT_RIGHT) return set_err(s, E2D_EINVAL, "bad layout");
  const size_t n = 4 * cells(s);
  double *src = nullptr;
  int rc = fp64_view(s, which, &src);
  if (rc != E2D_OK) return rc;
  if (layout == E2D_LAYOUT_LEFT) {
    E2D_CK(s, cudaMemcpyAsync(host, src, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream), "get_state copy");
    E2D_CK(s, cudaStreamSynchronize(s->stream), "get_state sync");
  } else {
    std::vector<double> tmp(n);
    E2D_CK(s, cudaMemcpyAsync(tmp.data(), src, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream), "get_state copy");
    E2D_CK(s, cudaStreamSynchronize(s->stream), "get_state sync");
    left_to_right(s->p, tmp.data(), host);
  }
  return E2D_OK;
}

int e2d_write_vtk(const e2d_params *pin, const double *host, int layout, const char *filename) {
  if (!pin || !host || !filename) return E2D_EINVAL;
  if (layout != E2D_LAYOUT_LEFT && layout != E2D_LAYOUT_RIGHT) return E2D_EINVAL;
  const e2d_params &p = *pin;
  if (p.isize != p.nx + 4 || p.jsize != p.ny + 4 || p.nx < 1 || p.ny < 1) return E2D_EINVAL;
  FILE *f = std::fopen(filename, "w");
  if (!f) return E2D_EIO;
  // text layout of src/HydroRun.h:546-607; numbers in the default ostream
  // format, which is printf's %g (6 significant digits)
  static const char *names[4] = {"rho", "E", "mx", "my"};
  const int one = 1;
  const bool big = (*(const char *)&one) == 0;
  std::fprintf(f, "<?xml version=\"1.0\"?>\n");
  std::fprintf(f, "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"%s\">\n",
               big ? "BigEndian" : "LittleEndian");
  std::fprintf(f, "  <ImageData WholeExtent=\"0 %d 0 %d 0 0\" Origin=\"%g %g 0\" Spacing=\"%g %g 0\">\n",
               p.nx, p.ny, p.xmin, p.ymin, p.dx, p.dy);
  std::fprintf(f, "  <Piece Extent=\"0 %d 0 %d 0 0 \">\n", p.nx, p.ny);
  std::fprintf(f, "    <PointData>\n    </PointData>\n    <CellData>\n");
  const size_t plane = (size_t)p.isize * p.jsize;
  for (int v = 0; v < 4; ++v) {
    std::fprintf(f, "    <DataArray type=\"Float64\" Name=\"%s\" format=\"ascii\" >\n", names[v]);
    // interior cells, i fastest (the reference's LayoutLeft index order)
    for (int j = 2; j <= p.jsize - 3; ++j)
      for (int i = 2; i <= p.isize - 3; ++i) {
        const size_t k = layout == E2D_LAYOUT_LEFT ? i + (size_t)p.isize * j + plane * v
                                                   : ((size_t)i * p.jsize + j) * 4 + v;
        std::fprintf(f, "%g ", host[k]);
      }
    std::fprintf(f, "\n    </DataArray>\n");
  }
  std::fprintf(f, "    </CellData>\n  </Piece>\n  </ImageData>\n</VTKFile>\n");
  const bool ok = std::ferror(f) == 0;
  return (std::fclose(f) == 0 && ok) ? E2D_OK : E2D_EIO;
}

int e2d_save_vtk(e2d_sim *s, int which, const char *filename) {
  if (!s || !filename || (which != 0 && which != 1)) return set_err(s, E2D_EINVAL, "bad save_vtk args");
  std::vector<double> host(4 * cells(s));
  int rc = e2d_get_state(s, which, host.data(), E2D_LAYOUT_LEFT);
  if (rc != E2D_OK) return rc;
  rc = e2d_write_vtk(&s->p, host.data(), E2D_LAYOUT_LEFT, filename);
  if (rc == E2D_EIO) return set_err(s, E2D_EIO, std::string("cannot write ") + filename);
  return rc;
}

int e2d_make_boundaries(e2d_sim *s, int which) {
  if (!s || (which != 0 && which != 1)) return set_err(s, E2D_EINVAL, "bad make_boundaries args");
  s->q_ready = -1;
  // FP32C states keep no ghost cells: every reader maps them on the fly
  if (s->fp32) return E2D_OK;
  E2D_CK(s, launch_fill_f64(s->kp, s->U[which], nullptr, nullptr, s->clk, FILL_GHOSTS_IN, s->stream), "make_boundaries");
  return E2D_OK;
}

int e2d_compute_dt(e2d_sim *s, int useU, double *dt) {
  if (!s || !dt) return set_err(s, E2D_EINVAL, "bad compute_dt args");
  const int which = (useU == 0) ? 0 : 1;
  E2D_CK(s, cudaMemsetAsync(&s->clk->invdt_bits, 0, sizeof(unsigned long long), s->stream), "dt reset");
  E2D_CK(s, cudaMemsetAsync(&s->clk->status, 0, sizeof(unsigned int), s->stream), "dt reset");
  if (s->fp32)
    E2D_CK(s, launch_f32c_dt(s->kp32, s->W[which], s->clk, -1, s->stream), "compute_dt");
  else
    E2D_CK(s, launch_fill_f64(s->kp, s->U[which], nullptr, nullptr, s->clk, FILL_DT, s->stream), "compute_dt");
  E2D_CK(s, cudaMemcpyAsync(s->clk_host, s->clk, sizeof(DevClock), cudaMemcpyDeviceToHost, s->stream), "dt copy");
  E2D_CK(s, cudaStreamSynchronize(s->stream), "dt sync");
  double inv;
  std::memcpy(&inv, &s->clk_host->invdt_bits, sizeof(double));
  *dt = s->p.cfl / inv;  // src/HydroRun.h:248
  if (s->clk_host->status & E2D_FLAG_NONFINITE) return set_err(s, E2D_ENUMERIC, "non-finite state value");
  return E2D_OK;
}

int e2d_godunov_unsplit(e2d_sim *s, int nStep, double dt) {
  if (!s) return E2D_EINVAL;
  if (s->kp.fast) return set_err(s, E2D_EINVAL, "fp64_fast runs through the device time loop (e2d_step_n) only");
  s->q_ready = -1;
  const int par = (nStep % 2 == 0) ? 0 : 1;  // src/HydroRun.h:263-270
  if (s->fp32) {
    E2D_CK(s, launch_f32c_step(s->kp32, s->p.riemannSolverType, s->W[par], s->W[par ^ 1], s->TM[par], s->clk, 0, dt,
                               s->stream), "godunov step");
    return E2D_OK;
  }
  double *in = s->U[par], *out = s->U[par ^ 1];
  if (s->impl != 0) {  // src/HydroRun.h:332-360
    E2D_CK(s, launch_fill_f64(s->kp, in, out, s->Q[0], s->clk, FILL_WRITE_Q | FILL_GHOSTS_IN | FILL_COPY_OUT,
                              s->stream), "godunov primitives");
    E2D_CK(s, launch_impl12_f64(s->kp, s->impl, s->p.riemannSolverType, s->Q[0], out, s->impl_scratch, s->clk, 0,
                                dt, nullptr, s->stream), "godunov implementation 1/2");
    return E2D_OK;
  }
  const int mode = FILL_WRITE_Q | FILL_GHOSTS_IN | FILL_GHOSTS_OUT;
  E2D_CK(s, launch_fill_f64(s->kp, in, out, s->Q[0], s->clk, mode, s->stream), "godunov primitives");
  E2D_CK(s, launch_flux_update_f64(s->kp, s->p.riemannSolverType, s->Q[0], in, out, s->clk, 0, dt,
                                   nullptr, s->stream), "godunov fluxes");
  return E2D_OK;
}

int e2d_step_n(e2d_sim *s, int n, double t_end, double *t, int *nStep, double *dt_trace) {
  if (!s || !t || !nStep || n < 0) return set_err(s, E2D_EINVAL, "bad step_n args");
  if (n == 0) return E2D_OK;
  int rc = ensure_trace(s, n);
  if (rc != E2D_OK) return rc;
  DevClock c{};
  c.t = *t;
  c.t_end = t_end;
  c.nstep = *nStep;
  c.trace_base = *nStep;
  c.trace_cap = n;
  c.trace = s->dt_trace;
  const int par0 = (*nStep % 2 == 0) ? 0 : 1;
  // the fused FP64 step reads the primitives and CFL maximum of its input:
  // from the previous call when nothing has changed the state since, else
  // from a prologue fill
  const bool fused = !s->fp32 && !s->f64_split && s->impl == 0;
  const bool prologue = fused && s->q_ready != par0;
  if (fused && !prologue) c.acc[par0] = s->q_acc;
  s->q_ready = -1;
  *s->clk_host = c;
  E2D_CK(s, cudaMemcpyAsync(s->clk, s->clk_host, sizeof(DevClock), cudaMemcpyHostToDevice, s->stream), "clock upload");
  // FP32C and the fused FP64 step: the first step's CFL maximum (and the
  // primitives of the input state); later steps fold it in their epilogue
  if (s->fp32) E2D_CK(s, launch_f32c_dt(s->kp32, s->W[par0], s->clk, *nStep & 1, s->stream), "initial dt");
  if (s->profiling) {
    size_t ev = 0;
    std::vector<std::pair<std::string, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    const std::string rs = riemann_name(s->p.riemannSolverType);
    if (prologue) {
      cudaEvent_t a = pool_event(s, ev++), b = pool_event(s, ev++);
      if (!a || !b) return set_err(s, E2D_ECUDA, "event create");
      E2D_CK(s, cudaEventRecord(a, s->stream), "event");
      E2D_CK(s, enqueue_prologue(s, par0, *nStep), "prologue");
      E2D_CK(s, cudaEventRecord(b, s->stream), "event");
      marks.push_back({"k_fill_f64 (prologue)", {a, b}});
    }
    for (int k = 0; k < n; ++k) {
      const int par = (par0 + k) & 1;
      cudaEvent_t a = pool_event(s, ev++), b = pool_event(s, ev++), c2 = pool_event(s, ev++);
      if (!a || !b || !c2) return set_err(s, E2D_ECUDA, "event create");
      if (s->fp32) {
        E2D_CK(s, cudaEventRecord(a, s->stream), "event");
        E2D_CK(s, launch_f32c_step(s->kp32, s->p.riemannSolverType, s->W[par], s->W[par ^ 1], s->TM[par], s->clk, 1, 0.0,
                                   s->stream), "step");
        E2D_CK(s, cudaEventRecord(b, s->stream), "event");
        marks.push_back({"k_step_f32c<" + rs + ">", {a, b}});
        continue;
      }
      if (!s->f64_split) {
        E2D_CK(s, cudaEventRecord(a, s->stream), "event");
        E2D_CK(s, enqueue_step(s, par), "step");
        E2D_CK(s, cudaEventRecord(b, s->stream), "event");
        marks.push_back({s->impl ? "implementation " + std::to_string(s->impl) + " step<" + rs + ">"
                                 : "k_step_f64<" + rs + ">", {a, b}});
        continue;
      }
      double *in = s->U[par], *out = s->U[par ^ 1];
      E2D_CK(s, cudaEventRecord(a, s->stream), "event");
      E2D_CK(s, launch_fill_f64(s->kp, in, out, s->Q[0], s->clk,
                                FILL_WRITE_Q | FILL_GHOSTS_IN | FILL_GHOSTS_OUT | FILL_DT | FILL_DEVICE_CLOCK,
                                s->stream), "fill");
      E2D_CK(s, cudaEventRecord(b, s->stream), "event");
      E2D_CK(s, launch_flux_update_f64(s->kp, s->p.riemannSolverType, s->Q[0], in, out, s->clk, 1, 0.0,
                                       s->dt_trace, s->stream), "flux");
      E2D_CK(s, cudaEventRecord(c2, s->stream), "event");
      marks.push_back({"k_fill_f64", {a, b}});
      marks.push_back({"k_flux_update_f64<" + rs + ">", {b, c2}});
    }
    E2D_CK(s, cudaStreamSynchronize(s->stream), "profiled step sync");
    for (auto &m : marks) {
      float ms = 0.f;
      E2D_CK(s, cudaEventElapsedTime(&ms, m.second.first, m.second.second), "event time");
      record_kernel(s, m.first, ms);
    }
  } else {
    if (prologue) E2D_CK(s, enqueue_prologue(s, par0, *nStep), "prologue");
    int done = 0;
    while (n - done >= kGraphSteps) {
      cudaGraphExec_t g;
      rc = get_graph(s, kGraphSteps, (par0 + done) & 1, &g);
      if (rc != E2D_OK) return rc;
      E2D_CK(s, cudaGraphLaunch(g, s->stream), "graph launch");
      done += kGraphSteps;
    }
    for (; done < n; ++done) E2D_CK(s, enqueue_step(s, (par0 + done) & 1), "step launch");
  }
  E2D_CK(s, cudaMemcpyAsync(s->clk_host, s->clk, sizeof(DevClock), cudaMemcpyDeviceToHost, s->stream), "clock download");
  E2D_CK(s, cudaStreamSynchronize(s->stream), "step_n sync");
  const int taken = s->clk_host->nstep - *nStep;
  if (dt_trace && taken > 0)
    E2D_CK(s, cudaMemcpy(dt_trace, s->dt_trace, sizeof(double) * taken, cudaMemcpyDeviceToHost), "trace copy");
  *t = s->clk_host->t;
  *nStep = s->clk_host->nstep;
  if (s->clk_host->status & E2D_FLAG_TIMEOUT)
    return set_err(s, E2D_ETIMEOUT, "a staging wait gave up: the state of this call is incomplete");
  if (s->clk_host->status & (E2D_FLAG_NONFINITE | E2D_FLAG_BAD_DT))
    return set_err(s, E2D_ENUMERIC, (s->clk_host->status & E2D_FLAG_NONFINITE) ? "non-finite state value"
                                                                              : "non-positive or non-finite dt");
  if (fused) {  // the last step (or the prologue) left U[nStep & 1]'s primitives and CFL maximum
    s->q_ready = *nStep & 1;
    s->q_acc = s->clk_host->acc[*nStep & 1];
  }
  return E2D_OK;
}

int e2d_conservation(e2d_sim *s, int which, double sums[4]) {
  if (!s || !sums || (which != 0 && which != 1)) return set_err(s, E2D_EINVAL, "bad conservation args");
  double *u = nullptr;
  int rc = fp64_view(s, which, &u);
  if (rc != E2D_OK) return rc;
  E2D_CK(s, launch_sums_f64(s->kp.g, u, s->partial, s->red_out, s->stream), "conservation");
  E2D_CK(s, cudaMemcpyAsync(sums, s->red_out, sizeof(double) * 4, cudaMemcpyDeviceToHost, s->stream), "conservation copy");
  E2D_CK(s, cudaStreamSynchronize(s->stream), "conservation sync");
  return E2D_OK;
}

int e2d_l1_diff(e2d_sim *a, int wa, e2d_sim *b, int wb, int var, double *l1_diff, double *l1_ref) {
  if (!a || !b || !l1_diff || !l1_ref || var < 0 || var > 3 || (wa != 0 && wa != 1) || (wb != 0 && wb != 1))
    return set_err(a, E2D_EINVAL, "bad l1_diff args");
  if (a->p.nx != b->p.nx || a->p.ny != b->p.ny) return set_err(a, E2D_EINVAL, "l1_diff: grids differ");
  if (a == b && a->fp32) return set_err(a, E2D_EINVAL, "l1_diff: one FP32C handle has one staging array");
  double *ua = nullptr, *ub = nullptr;
  int rc = fp64_view(a, wa, &ua);
  if (rc != E2D_OK) return rc;
  E2D_CK(a, cudaStreamSynchronize(a->stream), "l1 sync");
  rc = fp64_view(b, wb, &ub);
  if (rc != E2D_OK) return rc;
  E2D_CK(b, cudaStreamSynchronize(b->stream), "l1 sync");
  E2D_CK(a, launch_l1diff_f64(a->kp.g, ua, ub, var, a->partial, a->red_out, a->stream), "l1_diff");
  double r[2];
  E2D_CK(a, cudaMemcpyAsync(r, a->red_out, sizeof(r), cudaMemcpyDeviceToHost, a->stream), "l1 copy");
  E2D_CK(a, cudaStreamSynchronize(a->stream), "l1 sync");
  *l1_diff = r[0];
  *l1_ref = r[1];
  return E2D_OK;
}

int e2d_radial_profile(e2d_sim *s, int which, int nbins, double *distances, double *profile,
                       long long *counts) {
  if (!s || !distances || !profile || (which != 0 && which != 1))
    return set_err(s, E2D_EINVAL, "bad radial_profile args");
  const e2d_params &p = s->p;
  if (nbins <= 0) nbins = p.blast_nbins;
  if (nbins <= 0 || nbins > (1 << 24)) return set_err(s, E2D_EINVAL, "radial_profile: nbins out of range");
  // src/ComputeRadialProfileFunctor.h:90-103
  ProfileGeom g;
  g.xmin = p.xmin;
  g.ymin = p.ymin;
  g.dx = p.dx;
  g.dy = p.dy;
  g.cx = (p.xmin + p.xmax) / 2;
  g.cy = (p.ymin + p.ymax) / 2;
  const double Dx = (p.xmax - p.xmin) / 2;
  const double Dy = (p.ymax - p.ymin) / 2;
  g.rmax = std::sqrt(Dx * Dx + Dy * Dy);
  g.isize = p.isize;
  g.jsize = p.jsize;
  g.ghost = p.ghostWidth;
  g.nbins = nbins;
  double *u = nullptr;
  int rc = fp64_view(s, which, &u);
  if (rc != E2D_OK) return rc;
  const size_t words = 1 + 4 * (size_t)nbins;
  unsigned long long *scratch = nullptr;
  unsigned int *flags = nullptr;
  E2D_CK(s, cudaMallocAsync((void **)&scratch, sizeof(unsigned long long) * words + 16, s->stream), "profile alloc");
  flags = reinterpret_cast<unsigned int *>(scratch + words);
  std::vector<unsigned long long> host(words);
  unsigned int hflags = 0;
  cudaError_t e = launch_radial_profile(g, u, scratch, flags, s->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(host.data(), scratch, sizeof(unsigned long long) * words, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hflags, flags, sizeof hflags, cudaMemcpyDeviceToHost, s->stream);
  cudaFreeAsync(scratch, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return set_err(s, E2D_ECUDA, std::string("radial_profile: ") + cudaGetErrorString(e));
  if (hflags) return set_err(s, E2D_ENUMERIC, "radial_profile: non-finite density");
  finish_radial_profile(g, host.data(), profile, counts);
  const double dr = g.rmax / nbins;  // src/ComputeRadialProfileFunctor.h:121-127
  for (int b = 0; b < nbins; ++b) distances[b] = (b + 0.5) * dr;
  return E2D_OK;
}

int e2d_save_npy(const char *path, const double *data, long long n) {
  if (!path || (!data && n > 0) || n < 0) return E2D_EINVAL;
  // dictionary padded with spaces so that 10 + its length is a multiple of
  // 16, last byte '\n' (a full 16 spaces when it already is)
  const int one = 1;
  const char order = *reinterpret_cast<const char *>(&one) ? '<' : '>';
  std::string dict = std::string("{'descr': '") + order + "f8', 'fortran_order': False, 'shape': (" +
                     std::to_string(n) + ",), }";
  const int pad = 16 - (int)((10 + dict.size()) % 16);
  dict.append(pad, ' ');
  dict.back() = '\n';
  std::string head = "\x93NUMPY";
  head.push_back('\x01');
  head.push_back('\x00');
  const unsigned short hl = (unsigned short)dict.size();
  head.push_back((char)(hl & 0xff));
  head.push_back((char)(hl >> 8));
  FILE *f = std::fopen(path, "wb");
  if (!f) return E2D_EIO;
  bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size() &&
            std::fwrite(dict.data(), 1, dict.size(), f) == dict.size() &&
            (n == 0 || std::fwrite(data, sizeof(double), (size_t)n, f) == (size_t)n);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? E2D_OK : E2D_EIO;
}

int e2d_eval_device(const e2d_params *pin, int what, int n, const double *in, double *out,
                    double dtdx, double dtdy) {
  if (!pin || !in || !out || n < 0 || what < E2D_EVAL_PRIMITIVES || what > E2D_EVAL_RIEMANN_HLLC)
    return E2D_EINVAL;
  if (n == 0) return E2D_OK;
  e2d_params p = *pin;
  const int rc = params_init(&p, nullptr);
  if (rc != E2D_OK) return rc;
  KParams64 kp;
  make_kparams(p, &kp);
  const int in_w = what == E2D_EVAL_PRIMITIVES ? 4 : what == E2D_EVAL_SLOPES ? 20
                   : what <= E2D_EVAL_TRACE_YMAX ? 12 : 8;
  const int out_w = what == E2D_EVAL_PRIMITIVES ? 5 : what == E2D_EVAL_SLOPES ? 8 : 4;
  double *din = nullptr, *dout = nullptr;
  cudaStream_t st = nullptr;
  int status = E2D_OK;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return E2D_ECUDA;
  if (cudaMalloc(&din, sizeof(double) * in_w * (size_t)n) != cudaSuccess ||
      cudaMalloc(&dout, sizeof(double) * out_w * (size_t)n) != cudaSuccess) {
    status = E2D_ENOMEM;
  } else if (cudaMemcpyAsync(din, in, sizeof(double) * in_w * (size_t)n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
             launch_eval_f64(kp, what, n, din, dout, dtdx, dtdy, st) != cudaSuccess ||
             cudaMemcpyAsync(out, dout, sizeof(double) * out_w * (size_t)n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
             cudaStreamSynchronize(st) != cudaSuccess) {
    status = E2D_ECUDA;
  }
  if (din) cudaFree(din);
  if (dout) cudaFree(dout);
  cudaStreamDestroy(st);
  return status;
}

int e2d_set_profiling(e2d_sim *s, int on) {
  if (!s) return E2D_EINVAL;
  s->profiling = on != 0;
  return E2D_OK;
}

int e2d_kernel_times(e2d_sim *s, int max_kernels, const char **names, double *ms, long *launches,
                     int *n_kernels) {
  if (!s || !n_kernels) return E2D_EINVAL;
  int k = 0;
  for (const auto &nm : s->k_names) {
    if (k < max_kernels) {
      if (names) names[k] = nm.c_str();
      if (ms) ms[k] = s->k_ms[nm];
      if (launches) launches[k] = s->k_count[nm];
    }
    ++k;
  }
  *n_kernels = k;
  return E2D_OK;
}

int e2d_reset_kernel_times(e2d_sim *s) {
  if (!s) return E2D_EINVAL;
  s->k_ms.clear();
  s->k_count.clear();
  s->k_names.clear();
  return E2D_OK;
}

}  // extern "C"
