"""The C ABI on the CPU: the library loads, exports every entry point that
include/e2d.h declares, and its ini reader / HydroParams::setup reproduce the
reference's parameters (golden values from the reference's own ConfigMap and
HydroParams code).  No device work is launched here."""
import json
import os
import re

import pytest

import _cases as C
import euler2d_kokkos_gb300 as e2d

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "e2d.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(e2d_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = e2d.load_library()
    syms = header_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    # and the Python binding covers all of them
    assert set(syms) == set(e2d.SIGNATURES)


def test_abi_version_and_status_strings():
    L = e2d.load_library()
    assert L.e2d_abi_version() == e2d.ABI_VERSION == 2
    for s in range(7):
        assert L.e2d_status_string(s)


REF_TO_FIELD = {
    "nx": "nx", "ny": "ny", "isize": "isize", "jsize": "jsize", "dx": "dx", "dy": "dy",
    "gamma0": "gamma0", "gamma6": "gamma6", "cfl": "cfl", "slope_type": "slope_type",
    "smallr": "smallr", "smallc": "smallc", "smallp": "smallp", "smallpp": "smallpp",
    "tEnd": "tEnd", "nStepmax": "nStepmax", "bc_xmin": "boundary_type_xmin",
    "bc_xmax": "boundary_type_xmax", "bc_ymin": "boundary_type_ymin",
    "bc_ymax": "boundary_type_ymax", "riemann": "riemannSolverType", "problem": "problemType",
    "impl": "implementationVersion", "xmin": "xmin", "xmax": "xmax", "ymin": "ymin", "ymax": "ymax",
}


@pytest.mark.parametrize("name", ["plain", "formatting", "defaults", "shocked_bubble", "bad_impl", "quirks"])
def test_params_from_ini_match_reference(golden_dir, tmp_path, name):
    g = json.load(open(os.path.join(golden_dir, "params.json")))[name]
    path = C.write_ini(g["ini"], str(tmp_path), f"{name}.ini")
    p = e2d.HydroParams.from_ini(path)
    for ref_key, field in REF_TO_FIELD.items():
        got = getattr(p, field)
        want = g["params"][ref_key]
        assert float(got) == want, (ref_key, got, want)


def test_params_blast_and_bubble_values(tmp_path):
    text = C.ini_text(16, 16, problem="blast",
                      extra="[blast]\nradius=0.125\npressure_in=10\n[shocked_bubble]\nshock_loc=0.3\n")
    p = e2d.HydroParams.from_ini(C.write_ini(text, str(tmp_path)))
    assert p.blast_radius == C.f32(0.125) and p.blast_pressure_in == 10.0
    assert p.blast_density_out == C.f32(1.2)  # reference default
    assert p.blast_center_x == C.f32(0.5)     # (xmin+xmax)/2
    assert p.shock_loc == C.f32(0.3)


def test_params_four_quadrant_states(tmp_path):
    """Defaults: the reference's hard-coded Lax-Liu case 3 and split 0.8 as
    FP64 literals (src/HydroRunFunctors.h:1607-1622); keys rho_q, p_q, u_q,
    v_q and split_x/y override them through the ini's float rounding."""
    p = e2d.HydroParams.from_ini(C.write_ini(C.ini_text(16, 16, problem="four_quadrant"), str(tmp_path)))
    assert (p.fq_split_x, p.fq_split_y) == (0.8, 0.8)
    assert [list(r) for r in p.fq_state] == [[1.5, 1.5, 0.0, 0.0], [0.5323, 0.3, 1.206, 0.0],
                                             [0.138, 0.029, 1.206, 1.206], [0.5323, 0.3, 0.0, 1.206]]
    text = C.ini_text(16, 16, problem="four_quadrant",
                      extra="[four_quadrant]\nsplit_x=0.5\nrho_2=0.7\nv_3=-0.25\n")
    p = e2d.HydroParams.from_ini(C.write_ini(text, str(tmp_path), "b.ini"))
    assert p.fq_split_x == 0.5 and p.fq_split_y == 0.8
    assert p.fq_state[2][0] == C.f32(0.7) and p.fq_state[3][3] == -0.25
    assert p.fq_state[0][0] == 1.5


def test_params_validation():
    p = e2d.HydroParams()
    p.nx, p.ny = 16, 16
    p.init()
    for field, bad in [("slope_type", 3.0), ("nx", 1), ("boundary_type_xmin", 4), ("gamma0", 1.0),
                       ("cfl", 0.0), ("riemannSolverType", 5)]:
        q = p.copy()
        setattr(q, field, bad)
        with pytest.raises(e2d.E2DError) as ei:
            q.init()
        assert ei.value.status == 1


def test_missing_ini_is_eio(tmp_path):
    with pytest.raises(e2d.E2DError) as ei:
        e2d.HydroParams.from_ini(str(tmp_path / "nope.ini"))
    assert ei.value.status == 6


def test_make_params_matches_ini(tmp_path):
    text = C.ini_text(40, 24, bc=(2, 3, 3, 1), gamma0=1.666, cfl=0.7, riemann="hll")
    a = e2d.HydroParams.from_ini(C.write_ini(text, str(tmp_path)))
    b = e2d.make_params(40, 24, bc=(2, 3, 3, 1), gamma0=1.666, cfl=0.7, riemann="hll",
                        problem="implode", slope_type=2)
    for f in ("nx", "ny", "isize", "jsize", "dx", "dy", "gamma0", "cfl", "smallp", "smallpp",
              "gamma6", "riemannSolverType", "boundary_type_xmax"):
        assert getattr(a, f) == getattr(b, f), f


def test_header_is_plain_c(tmp_path):
    """include/e2d.h compiles as C11 (the boundary cgo, JNI and ctypes
    callers bind), and a C driver loop over its entry points type-checks."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "use_e2d.c"
    src.write_text("""
#include <stdlib.h>
#include "e2d.h"
int run(const char *ini) {
  e2d_params p; e2d_sim *sim;
  if (e2d_params_from_ini(ini, &p) != E2D_OK) return 1;
  if (e2d_create(&p, &sim) != E2D_OK || e2d_init_problem(sim) != E2D_OK) return 2;
  double t = 0; int nStep = 0;
  int rc = e2d_step_n(sim, p.nStepmax, p.tEnd, &t, &nStep, NULL);
  double *u = malloc(sizeof(double) * 4 * p.isize * p.jsize);
  e2d_get_state(sim, nStep % 2, u, E2D_LAYOUT_LEFT);
  e2d_batch *b;
  if (e2d_batch_create(E2D_RIEMANN_HLLC, (size_t)1 << 30, 16, &b) == E2D_OK) e2d_batch_destroy(b);
  free(u);
  e2d_destroy(sim);
  return rc;
}
""")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-fsyntax-only", "-I", inc, str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_mirror_compiles(tmp_path):
    """include/euler2d_gb300.hpp (the C++ mirror of ConfigMap, HydroParams,
    HydroRun, the radial profile and batches) compiles as C++17 with the
    reference's driver loop written against it."""
    import shutil
    import subprocess

    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    src = tmp_path / "use_mirror.cpp"
    src.write_text("""
#include "euler2d_gb300.hpp"
using namespace euler2d_gb300;
int main(int argc, char **argv) {
  ConfigMap configMap(argv[1]);
  HydroParams params;
  params.setup(configMap);
  HydroRun hydro(params, configMap);
  double t = 0, dt = hydro.compute_dt(0);
  int nStep = 0;
  hydro.make_boundaries(hydro.U);
  hydro.make_boundaries(hydro.U2);
  while (t < params.tEnd && nStep < params.nStepmax) {
    dt = hydro.compute_dt(nStep % 2);
    if (t + dt > params.tEnd) dt = params.tEnd - t;
    hydro.godunov_unsplit(nStep, dt);
    nStep++;
    t += dt;
  }
  ComputeRadialProfileFunctor::apply(hydro, hydro.U);
  Batch batch(size_t(1) << 30);
  const int id = batch.admit(params, 0.1);
  while (batch.run(16) > 0) {
  }
  bool active = true;
  if (batch.poll(id, &active) != E2D_OK) return 2;
  std::vector<double> u = batch.state(id, params);
  batch.release(id);
  return argc + (int)u.size() > 0 ? 0 : 1;
}
""")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-I", inc, str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_batch_instance_bytes_is_the_admission_arithmetic():
    """Pool bytes one admission takes (host arithmetic, no device): FP32C,
    two states of 8 float planes with the row pitch padded to 4 floats plus
    the FP64 staging array of the initial state; FP64, U, U2 and the
    primitives of each; each rounded to the pool's 256-byte blocks.  Invalid
    parameters give 0."""
    rnd = lambda b: (b + 255) // 256 * 256
    for nx, ny in [(64, 64), (100, 37), (1024, 512), (2, 2)]:
        isize, jsize = nx + 4, ny + 4
        pitch = (isize + 3) // 4 * 4
        p32 = e2d.make_params(nx, ny, precision=e2d.PRECISION_FP32C)
        assert e2d.Batch.instance_bytes(p32) == rnd(2 * 8 * pitch * jsize * 4) + rnd(4 * isize * jsize * 8)
        p64 = e2d.make_params(nx, ny, precision=e2d.PRECISION_FP64)
        assert e2d.Batch.instance_bytes(p64) == rnd(4 * 4 * isize * jsize * 8)
    bad = e2d.make_params(16, 16)
    bad.cfl = 0.0
    assert e2d.Batch.instance_bytes(bad) == 0
