// e2d_batch.cu -- batched solves: many independent simulations of uneven
// size resident in one device memory pool, advanced together by one kernel
// launch per iteration for the FP32C instances (k_batch_f32c) and one for
// the FP64 ones (k_batch_step_f64) with per-instance dt, replayed from CUDA
// graphs; admission by free pool bytes; strip height per size class and
// the kernel's register budget set by a measured autotuner.
#include "e2d_internal.h"

#include <algorithm>
#include <cstring>
#include <iterator>
#include <map>
#include <new>
#include <string>
#include <vector>

using namespace e2d;

namespace {

// First-fit allocator over one device range; blocks aligned to 256 bytes.
class PoolAllocator {
 public:
  void reset(size_t bytes) {
    free_.clear();
    if (bytes) free_[0] = bytes;
    size_ = bytes;
    used_ = 0;
  }
  bool alloc(size_t bytes, size_t *off) {
    bytes = round(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes;
        const size_t start = it->first + bytes;
        free_.erase(it);
        if (rest) free_[start] = rest;
        used_ += bytes;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = round(bytes);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto next = std::next(it);
    if (next != free_.end() && it->first + it->second == next->first) {
      it->second += next->second;
      free_.erase(next);
    }
    if (it != free_.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t free_bytes() const { return size_ - used_; }
  size_t largest_free() const {
    size_t m = 0;
    for (auto &kv : free_) m = std::max(m, kv.second);
    return m;
  }
  static size_t round(size_t b) { return (b + 255) & ~(size_t)255; }

 private:
  std::map<size_t, size_t> free_;
  size_t size_ = 0, used_ = 0;
};

struct HostInst {
  bool used = false;
  bool fp64 = false;  // an FP64 instance (BatchInst64 table), else FP32C
  e2d_params p{};
  size_t off = 0, bytes = 0;
  int size_class = 0;
  BatchInst mirror{};      // last downloaded copy of the device entry (FP32C)
  BatchInst64 mirror64{};  // (FP64)
  double t() const { return fp64 ? mirror64.t : mirror.t; }
  int nstep() const { return fp64 ? mirror64.nstep : mirror.nstep; }
  int active() const { return fp64 ? mirror64.active : mirror.active; }
  unsigned int status() const { return fp64 ? mirror64.status : mirror.status; }
};

int size_class_of(int nx, int ny) {
  const int s = std::max(nx, ny);
  return s <= 192 ? 0 : s <= 512 ? 1 : 2;
}

}  // namespace

struct e2d_batch {
  int riemann = E2D_RIEMANN_HLLC;
  int variant = 4;
  int strip_h[3] = {16, 32, 64};  // per size class
  cudaStream_t stream = nullptr;
  char *pool = nullptr;
  size_t pool_bytes = 0;
  PoolAllocator alloc;
  int max_inst = 0;
  std::vector<HostInst> slots;
  BatchInst *d_insts = nullptr;  // slot-indexed device table
  int *d_list = nullptr;         // [0, max_inst): slot of list entry k; then strip_begin (max_inst + 1)
  std::vector<int> list;         // slots of the current work list
  int total_strips = 0;
  BatchInst64 *d_insts64 = nullptr;  // slot-indexed FP64 table
  int *d_list64 = nullptr;           // slots (max_inst), then tile_begin (max_inst + 1)
  std::vector<int> list64;           // slots of the current FP64 work list
  int total_tiles = 0;
  int sm_count = 152;  // multiprocessors of the batch's device (the FP64 kernel's persistent grid)
  bool list_dirty = true;
  int grid = 0;
  std::map<int, cudaGraphExec_t> graphs;  // iterations -> graph of the current list
  std::string err;
  long long cell_updates = 0;  // interior cell-updates done by run calls
};

namespace {

int berr(e2d_batch *b, int status, const std::string &m) {
  if (b) b->err = m;
  return status;
}

#define B_CK(b, call, what)                                                                              \
  do {                                                                                                   \
    cudaError_t e__ = (call);                                                                            \
    if (e__ != cudaSuccess)                                                                              \
      return berr(b, e__ == cudaErrorMemoryAllocation ? E2D_ENOMEM : E2D_ECUDA,                          \
                  std::string(what) + ": " + cudaGetErrorString(e__));                                   \
  } while (0)

void drop_graphs(e2d_batch *b) {
  for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
}

size_t inst_bytes(const KParams32 &kp) { return (size_t)2 * 8 * kp.wplane * sizeof(float); }
// FP64 instance: U, U2 and the primitives of each
size_t inst_bytes64(const KGeom &g) { return (size_t)4 * 4 * g.plane * sizeof(double); }

int sync_mirrors(e2d_batch *b) {
  std::vector<BatchInst> tmp(b->max_inst);
  std::vector<BatchInst64> tmp64(b->max_inst);
  B_CK(b, cudaMemcpyAsync(tmp.data(), b->d_insts, sizeof(BatchInst) * b->max_inst, cudaMemcpyDeviceToHost,
                          b->stream), "table download");
  B_CK(b, cudaMemcpyAsync(tmp64.data(), b->d_insts64, sizeof(BatchInst64) * b->max_inst, cudaMemcpyDeviceToHost,
                          b->stream), "table download");
  B_CK(b, cudaStreamSynchronize(b->stream), "table sync");
  for (int k = 0; k < b->max_inst; ++k) {
    HostInst &h = b->slots[k];
    if (!h.used) continue;
    if (h.fp64)
      h.mirror64 = tmp64[k];
    else
      h.mirror = tmp[k];
  }
  return E2D_OK;
}

// The FP64 work list: used, active FP64 instances with their tiles.
int rebuild_list64(e2d_batch *b) {
  std::vector<int> list, tb;
  int nt = 0;
  for (int k = 0; k < b->max_inst; ++k) {
    HostInst &h = b->slots[k];
    if (!h.used || !h.fp64 || !h.mirror64.active) continue;
    list.push_back(k);
    tb.push_back(nt);
    nt += h.mirror64.ntiles;
  }
  tb.push_back(nt);
  if (!list.empty()) {
    const size_t m = (size_t)b->max_inst;
    B_CK(b, cudaMemcpyAsync(b->d_list64, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, b->stream),
         "list upload");
    B_CK(b, cudaMemcpyAsync(b->d_list64 + m, tb.data(), sizeof(int) * tb.size(), cudaMemcpyHostToDevice, b->stream),
         "tile list upload");
  }
  b->list64 = list;
  b->total_tiles = nt;
  return E2D_OK;
}

// The work list: used, active instances; each gets the strip height of its
// size class, lowered (to 16 rows at least) while the list has fewer strips
// than the grid has warps -- the tail of a batch, when a few large instances
// are left, would otherwise leave SMs idle.  Results do not depend on it.
int rebuild_list(e2d_batch *b) {
  std::vector<int> list, begin;
  const int per_sm = batch_blocks_per_sm(b->riemann, b->variant);
  const long long warps = 152LL * per_sm * 4;
  int shift = 0;
  for (;; ++shift) {
    long long n = 0;
    bool all_min = true;
    for (int k = 0; k < b->max_inst; ++k) {
      HostInst &h = b->slots[k];
      if (!h.used || h.fp64 || !h.mirror.active) continue;
      KParams32 kp = h.mirror.kp;
      kp.strip_h = std::max(16, ((b->strip_h[h.size_class] >> shift) / 16) * 16);
      all_min &= kp.strip_h == 16;
      n += strips_of(kp);
    }
    if (n >= warps || all_min) break;
  }
  int total = 0;
  for (int k = 0; k < b->max_inst; ++k) {
    HostInst &h = b->slots[k];
    if (!h.used || h.fp64 || !h.mirror.active) continue;
    const int sh = std::max(16, ((b->strip_h[h.size_class] >> shift) / 16) * 16);
    if (h.mirror.kp.strip_h != sh) {
      h.mirror.kp.strip_h = sh;
      h.mirror.nstrips = strips_of(h.mirror.kp);
      B_CK(b, cudaMemcpyAsync(&b->d_insts[k].kp.strip_h, &h.mirror.kp.strip_h, sizeof(int),
                              cudaMemcpyHostToDevice, b->stream), "strip_h upload");
      B_CK(b, cudaMemcpyAsync(&b->d_insts[k].nstrips, &h.mirror.nstrips, sizeof(int), cudaMemcpyHostToDevice,
                              b->stream), "nstrips upload");
    }
    list.push_back(k);
    begin.push_back(total);
    total += h.mirror.nstrips;
  }
  begin.push_back(total);
  if (!list.empty()) {
    B_CK(b, cudaMemcpyAsync(b->d_list, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, b->stream),
         "list upload");
    B_CK(b, cudaMemcpyAsync(b->d_list + b->max_inst, begin.data(), sizeof(int) * begin.size(),
                            cudaMemcpyHostToDevice, b->stream), "strip list upload");
  }
  {
    const int rc = rebuild_list64(b);
    if (rc != E2D_OK) return rc;
  }
  B_CK(b, cudaStreamSynchronize(b->stream), "list sync");
  b->list = list;
  b->total_strips = total;
  b->grid = std::max(1, std::min((total + 3) / 4, 152 * per_sm));
  drop_graphs(b);
  b->list_dirty = false;
  return E2D_OK;
}

int launch_iterations(e2d_batch *b, int iterations) {
  auto it = b->graphs.find(iterations);
  cudaGraphExec_t exec = nullptr;
  if (it == b->graphs.end()) {
    cudaGraph_t graph;
    B_CK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "capture");
    cudaError_t le = cudaSuccess;
    const int m = b->max_inst;
    for (int k = 0; k < iterations && le == cudaSuccess; ++k) {
      if (!b->list.empty())
        le = launch_batch_f32c(b->riemann, b->variant, b->d_insts, b->d_list, b->d_list + m, (int)b->list.size(),
                               b->total_strips, b->grid, b->stream);
      if (le == cudaSuccess && !b->list64.empty())
        le = launch_batch_f64(b->riemann, b->d_insts64, b->d_list64, b->d_list64 + m, (int)b->list64.size(),
                              b->total_tiles, b->sm_count, b->stream);
    }
    cudaError_t ee = cudaStreamEndCapture(b->stream, &graph);
    if (le != cudaSuccess || ee != cudaSuccess) return berr(b, E2D_ECUDA, "batch capture");
    cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return berr(b, E2D_ECUDA, "batch graph instantiate");
    b->graphs[iterations] = exec;
  } else {
    exec = it->second;
  }
  B_CK(b, cudaGraphLaunch(exec, b->stream), "batch launch");
  return E2D_OK;
}

// An FP64 instance: U (initial state from the host or the device
// initialiser), U2 = U, the primitives of each, primed once here (the
// prologue of the device loop); bit-identical to the single FP64 path step
// for step.
int admit64(e2d_batch *b, const e2d_params &p, double t_end, const double *u0, int slot, int *id) {
  KParams64 kp;
  make_kparams(p, &kp);
  const size_t need = inst_bytes64(kp.g);
  size_t off = 0;
  if (!b->alloc.alloc(need, &off)) return berr(b, E2D_ENOMEM, "admit: pool full");
  double *u0d = reinterpret_cast<double *>(b->pool + off);
  double *u1d = u0d + 4 * kp.g.plane;
  double *q0d = u1d + 4 * kp.g.plane;
  double *q1d = q0d + 4 * kp.g.plane;
  const size_t state_bytes = sizeof(double) * 4 * (size_t)kp.g.plane;
  auto undo = [&](int st, const char *m) {
    cudaStreamSynchronize(b->stream);
    b->alloc.release(off, need);
    return berr(b, st, m);
  };
  if (u0) {
    if (cudaMemcpyAsync(u0d, u0, state_bytes, cudaMemcpyHostToDevice, b->stream) != cudaSuccess)
      return undo(E2D_ECUDA, "admit: upload");
  } else if (launch_init_f64(kp, p, u0d, b->stream) != cudaSuccess) {
    return undo(E2D_ECUDA, "admit: init");
  }
  if (cudaMemcpyAsync(u1d, u0d, state_bytes, cudaMemcpyDeviceToDevice, b->stream) != cudaSuccess)
    return undo(E2D_ECUDA, "admit: copy");
  BatchInst64 I{};
  I.kp = kp;
  I.u[0] = u0d;
  I.u[1] = u1d;
  I.q[0] = q0d;
  I.q[1] = q1d;
  I.t = 0.0;
  I.t_end = t_end;
  I.active = I.t < I.t_end;
  batch_f64_shape(kp, &I.nbx, &I.nfill, &I.ntx, &I.ntiles);
  HostInst &h = b->slots[slot];
  if (cudaMemcpyAsync(&b->d_insts64[slot], &I, sizeof(I), cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
      launch_batch_prime_f64(&b->d_insts64[slot], I.nfill, b->stream) != cudaSuccess ||
      cudaMemcpyAsync(&I, &b->d_insts64[slot], sizeof(I), cudaMemcpyDeviceToHost, b->stream) != cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess)
    return undo(E2D_ECUDA, "admit: table upload");
  h.used = true;
  h.fp64 = true;
  h.p = p;
  h.off = off;
  h.bytes = need;
  h.size_class = size_class_of(p.nx, p.ny);
  h.mirror64 = I;
  b->list_dirty = true;
  *id = slot;
  return E2D_OK;
}

}  // namespace

extern "C" {

int e2d_batch_create(int riemann, size_t pool_bytes, int max_instances, e2d_batch **out) {
  if (!out || pool_bytes == 0 || max_instances <= 0 || riemann < 0 || riemann > 2) return E2D_EINVAL;
  *out = nullptr;
  e2d_batch *b = new (std::nothrow) e2d_batch();
  if (!b) return E2D_ENOMEM;
  b->riemann = riemann;
  b->max_inst = max_instances;
  b->slots.resize(max_instances);
  auto fail = [&](int st) {
    e2d_batch_destroy(b);
    return st;
  };
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(E2D_ECUDA);
  {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
      return fail(E2D_ECUDA);
    b->sm_count = sms;
  }
  if (cudaMalloc(&b->pool, pool_bytes) != cudaSuccess) return fail(E2D_ENOMEM);
  b->pool_bytes = pool_bytes;
  b->alloc.reset(pool_bytes);
  if (cudaMalloc(&b->d_insts, sizeof(BatchInst) * (size_t)max_instances) != cudaSuccess) return fail(E2D_ENOMEM);
  if (cudaMalloc(&b->d_list, sizeof(int) * (2 * (size_t)max_instances + 1)) != cudaSuccess) return fail(E2D_ENOMEM);
  if (cudaMalloc(&b->d_insts64, sizeof(BatchInst64) * (size_t)max_instances) != cudaSuccess) return fail(E2D_ENOMEM);
  if (cudaMalloc(&b->d_list64, sizeof(int) * (2 * (size_t)max_instances + 1)) != cudaSuccess) return fail(E2D_ENOMEM);
  if (cudaMemsetAsync(b->d_insts, 0, sizeof(BatchInst) * (size_t)max_instances, b->stream) != cudaSuccess ||
      cudaMemsetAsync(b->d_insts64, 0, sizeof(BatchInst64) * (size_t)max_instances, b->stream) != cudaSuccess)
    return fail(E2D_ECUDA);
  // shared-memory limits of the kernels (idempotent; a batch may be the
  // process's first handle)
  if (configure_f64_kernels() != cudaSuccess || configure_f32c_kernels() != cudaSuccess) return fail(E2D_ECUDA);
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return fail(E2D_ECUDA);
  *out = b;
  return E2D_OK;
}

int e2d_batch_destroy(e2d_batch *b) {
  if (!b) return E2D_EINVAL;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  if (b->pool) cudaFree(b->pool);
  if (b->d_insts) cudaFree(b->d_insts);
  if (b->d_list) cudaFree(b->d_list);
  if (b->d_insts64) cudaFree(b->d_insts64);
  if (b->d_list64) cudaFree(b->d_list64);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return E2D_OK;
}

const char *e2d_batch_last_error(const e2d_batch *b) { return b ? b->err.c_str() : "null handle"; }

int e2d_batch_free_bytes(const e2d_batch *b, size_t *free_bytes, size_t *largest) {
  if (!b) return E2D_EINVAL;
  if (free_bytes) *free_bytes = b->alloc.free_bytes();
  if (largest) *largest = b->alloc.largest_free();
  return E2D_OK;
}

size_t e2d_batch_instance_bytes(const e2d_params *pin) {
  if (!pin) return 0;
  e2d_params p = *pin;
  if (params_init(&p, nullptr) != E2D_OK || p.precision == E2D_PRECISION_FP64_FAST) return 0;
  KParams32 kp;
  make_kparams32(p, &kp);
  if (p.precision == E2D_PRECISION_FP64) return PoolAllocator::round(inst_bytes64(kp.g));
  return PoolAllocator::round(inst_bytes(kp)) + PoolAllocator::round(sizeof(double) * 4 * (size_t)kp.g.plane);
}

int e2d_batch_admit(e2d_batch *b, const e2d_params *pin, double t_end, const double *u0, int *id) {
  if (!b || !pin || !id) return E2D_EINVAL;
  e2d_params p = *pin;
  int rc = params_init(&p, nullptr);
  if (rc != E2D_OK) return berr(b, rc, "admit: invalid parameters");
  if (p.riemannSolverType != b->riemann) return berr(b, E2D_EINVAL, "admit: riemann solver differs from the batch's");
  if (p.precision == E2D_PRECISION_FP64_FAST)
    return berr(b, E2D_EINVAL, "admit: fp64_fast runs on single simulations only (e2d_step_n)");
  int slot = -1;
  for (int k = 0; k < b->max_inst; ++k)
    if (!b->slots[k].used) {
      slot = k;
      break;
    }
  if (slot < 0) return berr(b, E2D_ENOMEM, "admit: no free instance slot");
  if (p.precision == E2D_PRECISION_FP64) return admit64(b, p, t_end, u0, slot, id);
  KParams32 kp;
  make_kparams32(p, &kp);
  const int cls = size_class_of(p.nx, p.ny);
  kp.strip_h = b->strip_h[cls];
  kp.variant = b->variant;
  // two compensated states, plus a temporary FP64 array for the initial state
  const size_t need = inst_bytes(kp);
  const size_t stage_bytes = sizeof(double) * 4 * (size_t)kp.g.plane;
  size_t off = 0, soff = 0;
  if (!b->alloc.alloc(need, &off)) return berr(b, E2D_ENOMEM, "admit: pool full");
  if (!b->alloc.alloc(stage_bytes, &soff)) {
    b->alloc.release(off, need);
    return berr(b, E2D_ENOMEM, "admit: pool full (staging)");
  }
  float *w0 = reinterpret_cast<float *>(b->pool + off);
  float *w1 = w0 + 8 * kp.wplane;
  double *stage = reinterpret_cast<double *>(b->pool + soff);
  KParams64 k64;
  make_kparams(p, &k64);
  auto undo = [&](int st, const char *m) {
    cudaStreamSynchronize(b->stream);
    b->alloc.release(soff, stage_bytes);
    b->alloc.release(off, need);
    return berr(b, st, m);
  };
  if (u0) {
    if (cudaMemcpyAsync(stage, u0, stage_bytes, cudaMemcpyHostToDevice, b->stream) != cudaSuccess)
      return undo(E2D_ECUDA, "admit: upload");
  } else if (launch_init_f64(k64, p, stage, b->stream) != cudaSuccess) {
    return undo(E2D_ECUDA, "admit: init");
  }
  if (launch_f32c_from_f64(kp, stage, w0, b->stream) != cudaSuccess) return undo(E2D_ECUDA, "admit: convert");
  BatchInst I{};
  if (!encode_f32c_map(&I.tm[0], w0, kp) || !encode_f32c_map(&I.tm[1], w1, kp))
    return undo(E2D_ECUDA, "admit: TMA map");
  I.kp = kp;
  I.w[0] = w0;
  I.w[1] = w1;
  I.t = 0.0;
  I.t_end = t_end;
  I.par = 0;
  I.nstep = 0;
  I.nsx = (kp.g.nx + 59) / 60;
  I.nstrips = strips_of(kp);
  BatchInst *dI = &b->d_insts[slot];
  if (cudaMemcpyAsync(dI, &I, sizeof(I), cudaMemcpyHostToDevice, b->stream) != cudaSuccess)
    return undo(E2D_ECUDA, "admit: table upload");
  if (launch_f32c_dt_to(kp, w0, &dI->acc[0], &dI->status, b->stream) != cudaSuccess)
    return undo(E2D_ECUDA, "admit: dt");
  if (launch_batch_arm(dI, b->stream) != cudaSuccess) return undo(E2D_ECUDA, "admit: arm");
  HostInst &h = b->slots[slot];
  if (cudaMemcpyAsync(&h.mirror, dI, sizeof(BatchInst), cudaMemcpyDeviceToHost, b->stream) != cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess)
    return undo(E2D_ECUDA, "admit: sync");
  b->alloc.release(soff, stage_bytes);
  h.used = true;
  h.fp64 = false;
  h.p = p;
  h.off = off;
  h.bytes = need;
  h.size_class = cls;
  b->list_dirty = true;
  *id = slot;
  return E2D_OK;
}

int e2d_batch_release(e2d_batch *b, int id) {
  if (!b || id < 0 || id >= b->max_inst || !b->slots[id].used) return E2D_EINVAL;
  B_CK(b, cudaStreamSynchronize(b->stream), "release sync");
  HostInst &h = b->slots[id];
  b->alloc.release(h.off, h.bytes);
  h.used = false;
  BatchInst zero{};
  BatchInst64 zero64{};
  B_CK(b, cudaMemcpyAsync(&b->d_insts[id], &zero, sizeof(zero), cudaMemcpyHostToDevice, b->stream), "release");
  B_CK(b, cudaMemcpyAsync(&b->d_insts64[id], &zero64, sizeof(zero64), cudaMemcpyHostToDevice, b->stream), "release");
  B_CK(b, cudaStreamSynchronize(b->stream), "release sync");
  b->list_dirty = true;
  return E2D_OK;
}

int e2d_batch_query(e2d_batch *b, int id, double *t, int *nstep, int *active) {
  if (!b || id < 0 || id >= b->max_inst || !b->slots[id].used) return E2D_EINVAL;
  const HostInst &m = b->slots[id];
  if (t) *t = m.t();
  if (nstep) *nstep = m.nstep();
  if (active) *active = m.active();
  if (m.status() & E2D_FLAG_TIMEOUT) return berr(b, E2D_ETIMEOUT, "instance stopped: a row-staging wait gave up");
  if (m.status() & (E2D_FLAG_NONFINITE | E2D_FLAG_BAD_DT)) return berr(b, E2D_ENUMERIC, "instance hit NaN/Inf or a bad dt");
  return E2D_OK;
}

int e2d_batch_get_state(e2d_batch *b, int id, double *host, int layout) {
  if (!b || !host || id < 0 || id >= b->max_inst || !b->slots[id].used) return E2D_EINVAL;
  if (layout != E2D_LAYOUT_LEFT) return berr(b, E2D_EINVAL, "batch get_state: LayoutLeft only");
  HostInst &h = b->slots[id];
  B_CK(b, cudaStreamSynchronize(b->stream), "get sync");
  if (h.fp64) {
    const size_t bytes = sizeof(double) * 4 * (size_t)h.mirror64.kp.g.plane;
    B_CK(b, cudaMemcpyAsync(host, h.mirror64.u[h.mirror64.par], bytes, cudaMemcpyDeviceToHost, b->stream), "get_state");
    B_CK(b, cudaStreamSynchronize(b->stream), "get_state");
    return E2D_OK;
  }
  const KParams32 kp = h.mirror.kp;
  const size_t stage_bytes = sizeof(double) * 4 * (size_t)kp.g.plane;
  size_t soff = 0;
  if (!b->alloc.alloc(stage_bytes, &soff)) return berr(b, E2D_ENOMEM, "get_state: no pool room for staging");
  double *stage = reinterpret_cast<double *>(b->pool + soff);
  cudaError_t e = launch_f32c_to_f64(kp, h.mirror.w[h.mirror.par], stage, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, stage, stage_bytes, cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  b->alloc.release(soff, stage_bytes);
  if (e != cudaSuccess) return berr(b, E2D_ECUDA, "get_state");
  return E2D_OK;
}

int e2d_batch_run(e2d_batch *b, int iterations, int *n_active) {
  if (!b || iterations < 0) return E2D_EINVAL;
  if (b->list_dirty) {
    int rc = rebuild_list(b);
    if (rc != E2D_OK) return rc;
  }
  if ((!b->list.empty() || !b->list64.empty()) && iterations > 0) {
    int rc = launch_iterations(b, iterations);
    if (rc != E2D_OK) return rc;
  }
  std::vector<int> before(b->max_inst);
  for (int k = 0; k < b->max_inst; ++k) before[k] = b->slots[k].nstep();
  int rc = sync_mirrors(b);
  if (rc != E2D_OK) return rc;
  int active = 0;
  for (int k = 0; k < b->max_inst; ++k) {
    HostInst &h = b->slots[k];
    if (!h.used) continue;
    b->cell_updates += (long long)(h.nstep() - before[k]) * h.p.nx * h.p.ny;
    if (h.active()) ++active;
  }
  for (int k : b->list)
    if (!b->slots[k].active()) b->list_dirty = true;
  for (int k : b->list64)
    if (!b->slots[k].active()) b->list_dirty = true;
  if (n_active) *n_active = active;
  return E2D_OK;
}

int e2d_batch_stream(e2d_batch *b, void **stream) {
  if (!b || !stream) return E2D_EINVAL;
  *stream = (void *)b->stream;
  return E2D_OK;
}

int e2d_batch_stats(e2d_batch *b, long long *cell_updates, int *n_used) {
  if (!b) return E2D_EINVAL;
  if (cell_updates) *cell_updates = b->cell_updates;
  if (n_used) {
    int n = 0;
    for (auto &h : b->slots) n += h.used ? 1 : 0;
    *n_used = n;
  }
  return E2D_OK;
}

int e2d_batch_set_tuning(e2d_batch *b, int variant, const int strip_h[3]) {
  if (!b) return E2D_EINVAL;
  if (variant >= 0 && variant < kF32cVariants) b->variant = variant;
  // strip heights are whole CFL fold units (16 rows)
  if (strip_h)
    for (int c = 0; c < 3; ++c)
      if (strip_h[c] > 0 && strip_h[c] <= 512) b->strip_h[c] = (strip_h[c] + 15) / 16 * 16;
  b->list_dirty = true;
  return E2D_OK;
}

int e2d_batch_get_tuning(const e2d_batch *b, int *variant, int strip_h[3]) {
  if (!b) return E2D_EINVAL;
  if (variant) *variant = b->variant;
  if (strip_h)
    for (int c = 0; c < 3; ++c) strip_h[c] = b->strip_h[c];
  return E2D_OK;
}

// Measured tuning on the live batch: strip height and register budget change
// how the work is cut, not one bit of any result (every cell is computed by
// the same expressions; the CFL fold is exact), so the iterations spent
// timing candidates are ordinary progress of the batch.
int e2d_batch_autotune(e2d_batch *b, int iters_per_trial) {
  if (!b || iters_per_trial <= 0) return E2D_EINVAL;
  cudaEvent_t e0, e1;
  B_CK(b, cudaEventCreate(&e0), "event");
  B_CK(b, cudaEventCreate(&e1), "event");
  auto trial = [&](double *ms_per_cell) -> int {
    int rc = rebuild_list(b);
    if (rc != E2D_OK) return rc;
    if (b->list.empty()) {
      *ms_per_cell = 0;
      return E2D_OK;
    }
    long long before = b->cell_updates;
    // one untimed launch builds the graph
    rc = launch_iterations(b, iters_per_trial);
    if (rc == E2D_OK) rc = e2d_batch_run(b, 0, nullptr);
    if (rc != E2D_OK) return rc;
    before = b->cell_updates;
    if (b->list_dirty) rc = rebuild_list(b);
    if (rc != E2D_OK || b->list.empty()) {
      *ms_per_cell = 0;
      return rc;
    }
    B_CK(b, cudaEventRecord(e0, b->stream), "event");
    rc = launch_iterations(b, iters_per_trial);
    if (rc != E2D_OK) return rc;
    B_CK(b, cudaEventRecord(e1, b->stream), "event");
    rc = e2d_batch_run(b, 0, nullptr);
    if (rc != E2D_OK) return rc;
    float ms = 0.f;
    B_CK(b, cudaEventElapsedTime(&ms, e0, e1), "event time");
    const long long done = b->cell_updates - before;
    *ms_per_cell = done > 0 ? ms / (double)done : 1e30;
    return E2D_OK;
  };
  int rc = E2D_OK;
  // register budget first, then each size class's strip height.  Only the
  // staged variants are timed: the register variants 0-3 measured 31-45
  // Gcell/s against 55-64 for the staged ones at every size tried, and each
  // trial costs a graph capture and four iterations of the live batch.
  static const int kTuned[] = {4, 5, 6};
  double best_ms = 1e30;
  int best_v = b->variant;
  for (int t = 0; t < 3 && rc == E2D_OK; ++t) {
    const int v = kTuned[t];
    b->variant = v;
    double ms;
    rc = trial(&ms);
    if (rc == E2D_OK && ms > 0 && ms < best_ms) best_ms = ms, best_v = v;
  }
  b->variant = best_v;
  static const int cand[3] = {16, 32, 64};
  for (int c = 0; c < 3 && rc == E2D_OK; ++c) {
    bool present = false;
    for (auto &h : b->slots) present |= h.used && !h.fp64 && h.mirror.active && h.size_class == c;
    if (!present) continue;
    int best_h = b->strip_h[c];
    double bm = 1e30;
    for (int k = 0; k < 3 && rc == E2D_OK; ++k) {
      b->strip_h[c] = cand[k];
      double ms;
      rc = trial(&ms);
      if (rc == E2D_OK && ms > 0 && ms < bm) bm = ms, best_h = cand[k];
    }
    b->strip_h[c] = best_h;
  }
  b->list_dirty = true;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

}  // extern "C"
