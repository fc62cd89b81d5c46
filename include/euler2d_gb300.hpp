// euler2d_gb300.hpp -- C++ host interface of the GB300 euler2d step,
// header-only over the C ABI of e2d.h.
//
// It keeps the names and argument meaning of the reference's driver API so a
// user of euler2d_kokkos can switch by changing the include and namespace:
//   ConfigMap         config/ConfigMap.h:25-47 (constructed from an ini path)
//   HydroParams       src/HydroParams.h:155-265 (setup / init / print)
//   HydroRun          src/HydroRun.h:44-134 (compute_dt / godunov_unsplit /
//                     make_boundaries, public U / U2 / Uhost)
// Differences: errors throw euler2d_gb300::Error instead of exit()/silent
// fallbacks; DataArray is a device view of one of the handle's two states.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "e2d.h"

namespace euler2d_gb300 {

using real_t = double;

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string &what)
      : std::runtime_error(what + ": " + e2d_status_string(status)), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status, const char *what, const e2d_sim *sim = nullptr) {
  if (status != E2D_OK) {
    std::string w(what);
    if (sim) w += std::string(" (") + e2d_last_error(sim) + ")";
    throw Error(status, w);
  }
}

// ConfigMap: holds the ini path; values are read by HydroParams::setup with
// the reference's ConfigMap semantics (strtof reals, case-insensitive keys).
// The getters are ConfigMap's / INIReader's (config/ConfigMap.h:25-47,
// config/inih/INIReader.h): strings, strtol base-0 integers, strtof reals,
// 1/yes/true/on and 0/no/false/off booleans, defaults for absent keys.
class ConfigMap {
 public:
  explicit ConfigMap(std::string filename) : filename_(std::move(filename)) {}
  const std::string &filename() const { return filename_; }
  std::string getString(const std::string &section, const std::string &name,
                        const std::string &default_value) const {
    std::vector<char> buf(4096);
    if (e2d_ini_get_string(filename_.c_str(), section.c_str(), name.c_str(), default_value.c_str(),
                           buf.data(), buf.size()) != E2D_OK)
      return default_value;
    return std::string(buf.data());
  }
  long getInteger(const std::string &section, const std::string &name, long default_value) const {
    const std::string v = getString(section, name, "");
    char *end = nullptr;
    const long n = std::strtol(v.c_str(), &end, 0);
    return end > v.c_str() ? n : default_value;
  }
  float getFloat(const std::string &section, const std::string &name, float default_value) const {
    const std::string v = getString(section, name, "");
    char *end = nullptr;
    const float x = std::strtof(v.c_str(), &end);
    return end > v.c_str() ? x : default_value;
  }
  bool getBool(const std::string &section, const std::string &name, bool default_value) const {
    const std::string v = getString(section, name, "");
    if (v == "1" || v == "yes" || v == "true" || v == "on") return true;
    if (v == "0" || v == "no" || v == "false" || v == "off") return false;
    return default_value;
  }

 private:
  std::string filename_;
};

struct HydroParams : public e2d_params {
  HydroParams() { e2d_params_defaults(this); }
  void setup(ConfigMap &map) { check(e2d_params_from_ini(map.filename().c_str(), this), "HydroParams::setup"); }
  void init() { check(e2d_params_init(this), "HydroParams::init"); }
  void print() const {
    std::printf("##########################\n");
    std::printf("Simulation run parameters:\n");
    std::printf("##########################\n");
    std::printf("nx         : %d\n", nx);
    std::printf("ny         : %d\n", ny);
    std::printf("dx         : %f\n", dx);
    std::printf("dy         : %f\n", dy);
    std::printf("imin       : %d\n", imin);
    std::printf("imax       : %d\n", imax);
    std::printf("jmin       : %d\n", jmin);
    std::printf("jmax       : %d\n", jmax);
    std::printf("nStepmax   : %d\n", nStepmax);
    std::printf("tEnd       : %f\n", tEnd);
    std::printf("nOutput    : %d\n", nOutput);
    std::printf("gamma0     : %f\n", gamma0);
    std::printf("cfl        : %f\n", cfl);
    std::printf("smallr     : %12.10f\n", smallr);
    std::printf("smallc     : %12.10f\n", smallc);
    std::printf("slope_type : %f\n", slope_type);
    std::printf("riemann    : %d\n", riemannSolverType);
    std::printf("problem    : %d\n", problemType);
    std::printf("implementation version : %d\n", implementationVersion);
    std::printf("precision  : %s\n", precision == E2D_PRECISION_FP64 ? "fp64" : "fp32c");
    std::printf("##########################\n");
  }
};

// Device view of one state of a HydroRun (LayoutLeft, 4 planes).
struct DataArray {
  double *data = nullptr;
  int isize = 0, jsize = 0;
  int which = 0;  // 0: U, 1: U2
  size_t size() const { return (size_t)4 * isize * jsize; }
};

class HydroRun {
 public:
  // src/HydroRun.h:143-216: allocate the states and set the initial condition.
  HydroRun(HydroParams &params, ConfigMap &configMap) : params(params), configMap(configMap) {
    check(e2d_create(&params, &sim_), "HydroRun");
    check(e2d_get_params(sim_, &params), "HydroRun");
    check(e2d_init_problem(sim_), "HydroRun init", sim_);
    U = view(0);
    U2 = view(1);
  }
  HydroRun(const HydroRun &) = delete;
  HydroRun &operator=(const HydroRun &) = delete;
  virtual ~HydroRun() {
    if (sim_) e2d_destroy(sim_);
  }

  HydroParams &params;
  ConfigMap &configMap;
  DataArray U, U2;
  std::vector<double> Uhost;  // host mirror filled by copy_to_host

  // src/HydroRun.h:227-251
  real_t compute_dt(int useU) {
    double dt = 0;
    check(e2d_compute_dt(sim_, useU, &dt), "compute_dt", sim_);
    return dt;
  }
  // src/HydroRun.h:258-272
  void godunov_unsplit(int nStep, real_t dt) {
    check(e2d_godunov_unsplit(sim_, nStep, dt), "godunov_unsplit", sim_);
  }
  // src/HydroRun.h:388-399
  void make_boundaries(const DataArray &Udata) {
    check(e2d_make_boundaries(sim_, Udata.which), "make_boundaries", sim_);
  }
  // the time loop of src/main.cpp:100-145 on the device, n steps at most
  int step_n(int n, real_t tEnd, real_t &t, int &nStep, double *dt_trace = nullptr) {
    const int before = nStep;
    check(e2d_step_n(sim_, n, tEnd, &t, &nStep, dt_trace), "step_n", sim_);
    return nStep - before;
  }
  // deep_copy(Uhost, Udata) of src/HydroRun.h:522
  const std::vector<double> &copy_to_host(const DataArray &Udata) {
    Uhost.resize(Udata.size());
    check(e2d_get_state(sim_, Udata.which, Uhost.data(), E2D_LAYOUT_LEFT), "copy_to_host", sim_);
    return Uhost;
  }
  // src/HydroRun.h:486-495 (saveData; VTK only, HDF5 is not built) and
  // :506-609 (saveVTK): Udata as <outputDir>/<outputPrefix>_<iStep, 7
  // digits>.vti, the names read from the ini's [output] section.
  void saveData(const DataArray &Udata, int iStep, const std::string &name) {
    if (params.ioVTK) saveVTK(Udata, iStep, name);
  }
  void saveVTK(const DataArray &Udata, int iStep, const std::string & /*name*/) {
    char num[16];
    std::snprintf(num, sizeof(num), "%07d", iStep);
    const std::string fn = configMap.getString("output", "outputDir", "./") + "/" +
                           configMap.getString("output", "outputPrefix", "output") + "_" + num + ".vti";
    check(e2d_save_vtk(sim_, Udata.which, fn.c_str()), "saveVTK", sim_);
  }
  void copy_from_host(const DataArray &Udata, const std::vector<double> &host) {
    check(e2d_set_state(sim_, Udata.which, host.data(), E2D_LAYOUT_LEFT), "copy_from_host", sim_);
  }
  e2d_sim *sim() { return sim_; }

 private:
  DataArray view(int which) {
    DataArray d;
    check(e2d_device_state(sim_, which, &d.data), "device_state");
    d.isize = params.isize;
    d.jsize = params.jsize;
    d.which = which;
    return d;
  }
  e2d_sim *sim_ = nullptr;
};

// ComputeRadialProfileFunctor::apply (src/ComputeRadialProfileFunctor.h:83-134):
// the mean density of Udata in [blast] nbins rings about the box centre,
// written as sedov_blast_radial_distances.npy and
// sedov_blast_density_profile.npy in the working directory.
struct ComputeRadialProfileFunctor {
  static void apply(HydroRun &hydro, const DataArray &Udata) {
    const int nb = hydro.params.blast_nbins;
    std::vector<double> dist(nb > 0 ? nb : 0), prof(dist.size());
    check(e2d_radial_profile(hydro.sim(), Udata.which, nb, dist.data(), prof.data(), nullptr),
          "ComputeRadialProfileFunctor", hydro.sim());
    check(e2d_save_npy("sedov_blast_radial_distances.npy", dist.data(), (long long)dist.size()),
          "save sedov_blast_radial_distances.npy");
    check(e2d_save_npy("sedov_blast_density_profile.npy", prof.data(), (long long)prof.size()),
          "save sedov_blast_density_profile.npy");
  }
};

// Batched solves (e2d_batch_* in e2d.h; no counterpart in the reference):
// solves of uneven size, each FP32C or FP64 as its HydroParams say, resident
// in one device pool and advanced together with per-solve dt and t_end.
class Batch {
 public:
  explicit Batch(size_t pool_bytes, int max_instances = 1024, int riemann = E2D_RIEMANN_HLLC) {
    check(e2d_batch_create(riemann, pool_bytes, max_instances, &b_), "Batch");
  }
  Batch(const Batch &) = delete;
  Batch &operator=(const Batch &) = delete;
  ~Batch() {
    if (b_) e2d_batch_destroy(b_);
  }
  // admit a solve: u0 (LayoutLeft FP64, ghosts included) or nullptr to build
  // the parameters' initial condition on the device; returns its id
  int admit(const HydroParams &p, double t_end, const double *u0 = nullptr) {
    int id = -1;
    ck(e2d_batch_admit(b_, &p, t_end, u0, &id), "Batch::admit");
    return id;
  }
  // advance every active solve; returns how many are still active
  int run(int iterations) {
    int n = 0;
    ck(e2d_batch_run(b_, iterations, &n), "Batch::run");
    return n;
  }
  bool active(int id, double *t = nullptr, int *nstep = nullptr) {
    int a = 0;
    ck(e2d_batch_query(b_, id, t, nstep, &a), "Batch::query");
    return a != 0;
  }
  // like active() without throwing for a solve the batch stopped: returns
  // E2D_OK, E2D_ENUMERIC (non-finite state or dt) or E2D_ETIMEOUT (a
  // row-staging wait gave up); *active, *t, *nstep are filled in every case
  int poll(int id, bool *active, double *t = nullptr, int *nstep = nullptr) {
    int a = 0;
    const int rc = e2d_batch_query(b_, id, t, nstep, &a);
    if (rc != E2D_OK && rc != E2D_ENUMERIC && rc != E2D_ETIMEOUT) ck(rc, "Batch::poll");
    if (active) *active = a != 0;
    return rc;
  }
  std::vector<double> state(int id, const HydroParams &p) {
    std::vector<double> u((size_t)4 * p.isize * p.jsize);
    ck(e2d_batch_get_state(b_, id, u.data(), E2D_LAYOUT_LEFT), "Batch::get_state");
    return u;
  }
  void release(int id) { ck(e2d_batch_release(b_, id), "Batch::release"); }
  void autotune(int iters_per_trial = 2) { ck(e2d_batch_autotune(b_, iters_per_trial), "Batch::autotune"); }
  e2d_batch *handle() { return b_; }

 private:
  void ck(int status, const char *what) {
    if (status != E2D_OK) throw Error(status, std::string(what) + " (" + e2d_batch_last_error(b_) + ")");
  }
  e2d_batch *b_ = nullptr;
};

}  // namespace euler2d_gb300
