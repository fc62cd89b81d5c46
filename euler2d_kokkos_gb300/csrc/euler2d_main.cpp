// euler2d_gb300 -- command-line driver with the behaviour of the reference's
// src/main.cpp:24-212: read an ini file, build HydroParams and HydroRun, run
// the time loop (dt from the CFL condition, clamped at tEnd), write VTK
// output every nOutput steps, the Sedov radial profile (.npy) for blasts
// with total_energy_inside > 0, and report the timing and the
// "Mcell-updates/s" figure (ghost cells counted, src/main.cpp:202-203).
//
//   euler2d_gb300 file.ini [--host-loop]
//
// By default the loop runs on the device in chunks between progress lines and
// outputs (e2d_step_n, graph-replayed); --host-loop runs it on the host
// exactly as the reference does (compute_dt + godunov_unsplit every step).
// Both produce the same bits.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "euler2d_gb300.hpp"

using namespace euler2d_gb300;

static std::string ini_string(const std::string &ini, const char *sec, const char *key, const char *dflt) {
  char buf[1024];
  if (e2d_ini_get_string(ini.c_str(), sec, key, dflt, buf, sizeof(buf)) != E2D_OK) return dflt;
  return buf;
}

int main(int argc, char *argv[]) {
  if (argc < 2) {
    std::fprintf(stderr,
                 "Error: wrong number of argument; input filename must be "
                 "the only parameter on the command line\n");
    return EXIT_FAILURE;
  }
  bool host_loop = false;
  for (int k = 2; k < argc; ++k)
    if (!std::strcmp(argv[k], "--host-loop")) host_loop = true;

  try {
    const std::string input_file = argv[1];
    ConfigMap configMap(input_file);
    HydroParams params;
    params.setup(configMap);
    params.print();

    const std::string outDir = ini_string(input_file, "output", "outputDir", "./");
    const std::string outPrefix = ini_string(input_file, "output", "outputPrefix", "output");
    auto save = [&](HydroRun &h, int nStep) {
      if (!params.ioVTK) return;
      char num[16];
      std::snprintf(num, sizeof(num), "%07d", nStep);
      const std::string fn = outDir + "/" + outPrefix + "_" + num + ".vti";
      check(e2d_save_vtk(h.sim(), nStep % 2, fn.c_str()), "saveVTK", h.sim());
    };

    HydroRun hydro(params, configMap);
    double t = 0, dt = 0;
    int nStep = 0;
    dt = hydro.compute_dt(nStep % 2);
    hydro.make_boundaries(hydro.U);
    hydro.make_boundaries(hydro.U2);

    std::printf("Start computation....\n");
    const auto t0 = std::chrono::steady_clock::now();
    double io_s = 0;
    while (t < params.tEnd && nStep < params.nStepmax) {
      if (nStep % 10 == 0) std::printf("time step=%7d (dt=% 10.8f t=% 10.8f)\n", nStep, dt, t);
      if (params.enableOutput && params.nOutput > 0 && nStep % params.nOutput == 0) {
        const auto a = std::chrono::steady_clock::now();
        std::printf("Output results at time t=%g step %d dt=%g\n", t, nStep, dt);
        save(hydro, nStep);
        io_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
      }
      if (host_loop) {
        dt = hydro.compute_dt(nStep % 2);
        if (t + dt > params.tEnd) dt = params.tEnd - t;
        hydro.godunov_unsplit(nStep, dt);
        nStep++;
        t += dt;
      } else {
        // run up to the next progress line or output step on the device
        int n = 10 - nStep % 10;
        if (params.enableOutput && params.nOutput > 0) {
          const int to_out = params.nOutput - nStep % params.nOutput;
          if (to_out < n) n = to_out;
        }
        if (nStep + n > params.nStepmax) n = params.nStepmax - nStep;
        double trace[10];
        const int before = nStep;
        hydro.step_n(n, params.tEnd, t, nStep, trace);
        if (nStep > before) dt = trace[nStep - before - 1];
        if (nStep == before) break;
      }
    }
    if (params.enableOutput && params.nOutput > 0) {
      const auto a = std::chrono::steady_clock::now();
      std::printf("Output results at time t=%g step %d dt=%g\n", t, nStep, dt);
      save(hydro, nStep);
      io_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
    }
    const double t_tot = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // post-processing for the Sedov blast (src/main.cpp:175-179); like the
    // reference it reads U whatever the parity of the last step
    if (params.problemType == E2D_PROBLEM_BLAST && params.blast_total_energy_inside > 0)
      ComputeRadialProfileFunctor::apply(hydro, hydro.U);
    std::printf("total           time : %5.3f secondes\n", t_tot);
    std::printf("io              time : %5.3f secondes %5.2f%%\n", io_s, 100 * io_s / t_tot);
    std::printf("Perf                 : %10.2f number of Mcell-updates/s\n",
                1.0 * nStep * params.isize * params.jsize / t_tot * 1e-6);
    std::printf("Perf (interior)      : %10.4f Gcell-updates/s\n",
                1.0 * nStep * params.nx * params.ny / t_tot * 1e-9);
  } catch (const Error &e) {
    std::fprintf(stderr, "euler2d_gb300: %s\n", e.what());
    return EXIT_FAILURE;
  }
  return EXIT_SUCCESS;
}
