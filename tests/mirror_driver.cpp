// The reference's driver loop (src/main.cpp:76-145) written against the C++
// mirror include/euler2d_gb300.hpp, as a user of euler2d_kokkos would port
// their main(): ConfigMap + HydroParams::setup, HydroRun, compute_dt,
// make_boundaries, the dt clamp at tEnd, godunov_unsplit, saveData.
//
//   mirror_driver <ini> <step limit, -1: the ini's nStepmax> <result file>
//
// The result file holds nStep (int32), t (double), the dt of every step and
// the final state (LayoutLeft doubles, ghosts included); the final state is
// also written by saveData as the ini's [output] section names it.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "euler2d_gb300.hpp"

using namespace euler2d_gb300;

int main(int argc, char **argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s <ini> <step limit> <result file>\n", argv[0]);
    return 2;
  }
  try {
    ConfigMap configMap(argv[1]);
    HydroParams params;
    params.setup(configMap);
    const int limit = std::atoi(argv[2]);
    if (limit >= 0) params.nStepmax = limit;
    HydroRun hydro(params, configMap);
    real_t t = 0, dt = hydro.compute_dt(0);
    int nStep = 0;
    hydro.make_boundaries(hydro.U);
    hydro.make_boundaries(hydro.U2);
    std::vector<double> dts;
    while (t < params.tEnd && nStep < params.nStepmax) {
      dt = hydro.compute_dt(nStep % 2);
      if (t + dt > params.tEnd) dt = params.tEnd - t;
      dts.push_back(dt);
      hydro.godunov_unsplit(nStep, dt);
      nStep++;
      t += dt;
    }
    const DataArray &cur = (nStep % 2 == 0) ? hydro.U : hydro.U2;
    hydro.saveData(cur, nStep, "U");
    const std::vector<double> &u = hydro.copy_to_host(cur);
    FILE *f = std::fopen(argv[3], "wb");
    if (!f) return 3;
    const int ns = nStep;
    bool ok = std::fwrite(&ns, sizeof ns, 1, f) == 1 && std::fwrite(&t, sizeof t, 1, f) == 1 &&
              std::fwrite(dts.data(), sizeof(double), dts.size(), f) == dts.size() &&
              std::fwrite(u.data(), sizeof(double), u.size(), f) == u.size();
    ok = std::fclose(f) == 0 && ok;
    return ok ? 0 : 3;
  } catch (const Error &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
}
