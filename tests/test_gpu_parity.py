"""Parity of the CUDA path (through the C ABI) with the reference.

The FP64 path is bit-identical to the reference: every comparison here is
exact equality of FP64 bits (tolerance 0) -- against golden fixtures made by
the reference itself (tests/golden) and against the CPU oracle for cases the
reference cannot run (the HLL and approx solvers selected by the riemann key,
ragged and larger grids)."""
import hashlib
import json
import os

import numpy as np
import pytest

import _cases as C
import euler2d_kokkos_gb300 as e2d
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

CASES = sorted(C.run_cases().keys())


def hydro_from_text(text, tmp_path, name="case.ini", **override):
    p = e2d.HydroParams.from_ini(C.write_ini(text, str(tmp_path), name))
    for k, v in override.items():
        setattr(p, k, v)
    p.init()
    return e2d.HydroRun(p, init_problem=False)


def run_device_loop(h, u0, nsteps, tend, chunk=None):
    h.set_state(0, u0)
    h.set_state(1, u0)
    t, ns, trace = 0.0, 0, []
    chunk = chunk or nsteps
    while ns < nsteps and t < tend:
        t, ns, tr = h.step_n(min(chunk, nsteps - ns), tend, t, ns)
        trace.append(tr)
        if len(tr) == 0:
            break
    return h.current(ns), np.concatenate(trace), t, ns


@pytest.mark.parametrize("name", CASES)
def test_device_loop_matches_reference_bitwise(gpu_lib, runs, tmp_path, name):
    text = str(runs[f"{name}__ini"])
    nmax, tend = C.run_limits(text)
    nsteps = min(nmax, C.run_cases()[name]["nsteps"])
    with hydro_from_text(text, tmp_path) as h:
        u, dts, t, ns = run_device_loop(h, runs[f"{name}__u0"], nsteps, tend, chunk=13)
    assert ns == int(runs[f"{name}__nsteps"])
    assert np.array_equal(dts, runs[f"{name}__dt"]), "dt sequence differs"
    assert t == float(runs[f"{name}__t"])
    assert np.array_equal(u, runs[f"{name}__u"]), "state differs (ghosts included)"


@pytest.mark.parametrize("name", ["implode_diag", "blast_reflect", "mixed_bc_smooth", "tend_clamp"])
def test_host_driven_loop_matches_reference_bitwise(gpu_lib, runs, tmp_path, name):
    """src/main.cpp's loop on the host: compute_dt, clamp, godunov_unsplit."""
    text = str(runs[f"{name}__ini"])
    nmax, tend = C.run_limits(text)
    nsteps = min(nmax, C.run_cases()[name]["nsteps"])
    u0 = runs[f"{name}__u0"]
    with hydro_from_text(text, tmp_path) as h:
        h.set_state(0, u0)
        h.set_state(1, u0)
        h.make_boundaries(0)
        h.make_boundaries(1)
        t, ns, dts = 0.0, 0, []
        while t < tend and ns < nsteps:
            dt = h.compute_dt(ns % 2)
            if t + dt > tend:
                dt = tend - t
            dts.append(dt)
            h.godunov_unsplit(ns, dt)
            ns += 1
            t += dt
        u = h.current(ns)
    assert np.array_equal(np.array(dts), runs[f"{name}__dt"])
    assert np.array_equal(u, runs[f"{name}__u"])


@pytest.mark.parametrize("name", ["implode_ref_ini", "blast_reflect", "four_quadrant_absorb",
                                  "discontinuity_absorb", "shocked_bubble"])
def test_device_initial_conditions_match_reference(gpu_lib, runs, tmp_path, name):
    text = str(runs[f"{name}__ini"])
    p = e2d.HydroParams.from_ini(C.write_ini(text, str(tmp_path)))
    with e2d.HydroRun(p, init_problem=True) as h:
        assert np.array_equal(h.U, runs[f"{name}__u0"])
        assert np.array_equal(h.U2, runs[f"{name}__u0"])


def test_c1_implode_256_1000_steps(gpu_lib, golden_dir, tmp_path):
    g = json.load(open(os.path.join(golden_dir, "c1.json")))
    u0 = C.implode_diag_state(256, 256, C.f32(1.4))
    with hydro_from_text(g["ini"], tmp_path) as h:
        u, dts, t, ns = run_device_loop(h, u0, 1000, C.f32(10.0))
    assert ns == 1000
    assert [float(x).hex() for x in dts] == g["dt_hex"]
    assert hashlib.sha256(np.ascontiguousarray(u).tobytes()).hexdigest() == g["sha256_state"]


@pytest.mark.parametrize("tag", ["1111", "2222", "3333", "1231", "3123"])
def test_make_boundaries_and_compute_dt(gpu_lib, kat, tmp_path, tag):
    with hydro_from_text(str(kat[f"bc{tag}_ini"]), tmp_path) as h:
        h.set_state(0, kat[f"bc{tag}_u0"])
        h.set_state(1, kat[f"bc{tag}_u0"])
        assert h.compute_dt(0) == float(kat[f"bc{tag}_dt"])
        h.make_boundaries(1)
        assert np.array_equal(h.U2, kat[f"bc{tag}_u"])
        assert np.array_equal(h.U, kat[f"bc{tag}_u0"])  # the other state is untouched


@pytest.mark.parametrize("solver", ["hll", "approx", "hllc"])
@pytest.mark.parametrize("case", ["implode_diag", "four_quadrant_absorb", "periodic_smooth"])
def test_riemann_key_selects_solver_bitwise_vs_oracle(gpu_lib, runs, tmp_path, solver, case):
    """The riemann ini key selects the solver (the reference always runs
    HLLC); each choice is compared with the oracle's restatement."""
    text = str(runs[f"{case}__ini"]).replace("riemann=hllc", f"riemann={solver}")
    u0 = runs[f"{case}__u0"]
    kw = C.oracle_kwargs(text)
    p = po.make_params(**kw)
    uo, dto, to, no = po.run(p, u0, 25, C.f32(10.0))
    with hydro_from_text(text, tmp_path) as h:
        assert h.params.riemannSolverType == e2d.RIEMANN[solver]
        u, dts, t, ns = run_device_loop(h, u0, 25, C.f32(10.0))
    assert ns == no == 25
    assert np.array_equal(dts, dto)
    assert np.array_equal(u, uo)


@pytest.mark.parametrize("nx,ny,bc", [(2, 2, (1, 1, 1, 1)), (3, 5, (3, 3, 3, 3)), (37, 23, (1, 2, 3, 3)),
                                      (33, 17, (2, 2, 2, 2)), (31, 15, (3, 3, 1, 1)),
                                      (65, 64, (1, 1, 2, 2)), (100, 7, (2, 1, 3, 3))])
def test_ragged_sizes_bitwise_vs_oracle(gpu_lib, tmp_path, nx, ny, bc):
    g = C.f32(1.4)
    text = C.ini_text(nx, ny, bc=bc)
    u0 = C.smooth_state(nx, ny, g, seed=nx * 100 + ny, amp=0.3)
    p = po.make_params(**C.oracle_kwargs(text))
    uo, dto, _, no = po.run(p, u0, 12, C.f32(10.0))
    with hydro_from_text(text, tmp_path) as h:
        u, dts, _, ns = run_device_loop(h, u0, 12, C.f32(10.0), chunk=5)
    assert ns == no
    assert np.array_equal(dts, dto)
    assert np.array_equal(u, uo)


def test_larger_grid_bitwise_vs_oracle(gpu_lib, tmp_path):
    """512x384 blast (the 4096^2 benchmark case at reduced size), 20 steps."""
    text = C.ini_text(512, 384, problem="blast",
                      extra="[blast]\nradius=0.125\ncenter_x=0.5\ncenter_y=0.5\ndensity_in=1.0\n"
                            "density_out=1.0\npressure_in=10.0\npressure_out=0.1\n")
    path = C.write_ini(text, str(tmp_path))
    p = e2d.HydroParams.from_ini(path)
    with e2d.HydroRun(p) as h:
        u0 = h.U
        u, dts, _, ns = run_device_loop(h, u0, 20, C.f32(10.0), chunk=8)
    op = po.make_params(**C.oracle_kwargs(text))
    uo, dto, _, no = po.run(op, u0, 20, C.f32(10.0))
    assert np.array_equal(dts, dto)
    assert np.array_equal(u, uo)


def test_layout_right_round_trip(gpu_lib, tmp_path):
    text = C.ini_text(12, 9)
    u0 = C.smooth_state(12, 9, C.f32(1.4), seed=3)
    with hydro_from_text(text, tmp_path) as h:
        right = np.ascontiguousarray(np.transpose(u0, (2, 1, 0)))  # (isize, jsize, 4)
        h.set_state(0, right, layout=e2d.LAYOUT_RIGHT)
        assert np.array_equal(h.U, u0)
        back = h.get_state(0, layout=e2d.LAYOUT_RIGHT)
        assert np.array_equal(back, right)


def test_nonfinite_state_reports_enumeric(gpu_lib, tmp_path):
    """A NaN planted in the host state is reported as E2D_ENUMERIC by the
    device check; the context stays usable afterwards."""
    text = C.ini_text(16, 16)
    u0 = C.smooth_state(16, 16, C.f32(1.4), seed=9)
    u0[0, 8, 8] = np.nan
    with hydro_from_text(text, tmp_path) as h:
        h.set_state(0, u0)
        h.set_state(1, u0)
        with pytest.raises(e2d.E2DError) as ei:
            h.step_n(3, 10.0, 0.0, 0)
        assert ei.value.status == 3
    with hydro_from_text(text, tmp_path) as h2:  # still usable
        h2.set_state(0, C.smooth_state(16, 16, C.f32(1.4), seed=9))
        assert h2.compute_dt(0) > 0


def _kat_device_params(kat, key, tmp_path):
    return e2d.HydroParams.from_ini(C.write_ini(str(kat[key]), str(tmp_path), "kat.ini"))


def test_device_primitives_kat(gpu_lib, kat, tmp_path):
    p = _kat_device_params(kat, "ini_slope2", tmp_path)
    out = e2d.eval_device(p, "primitives", kat["prim_u"])
    assert np.array_equal(out[:, :4], kat["prim_q"])
    assert np.array_equal(out[:, 4], kat["prim_c"])


@pytest.mark.parametrize("st", [1, 2])
def test_device_slopes_kat(gpu_lib, kat, tmp_path, st):
    p = _kat_device_params(kat, f"ini_slope{st}", tmp_path)
    out = e2d.eval_device(p, "slopes", kat["slope_q5"])
    assert np.array_equal(out[:, :4], kat[f"slope{st}_dqx"])
    assert np.array_equal(out[:, 4:], kat[f"slope{st}_dqy"])


@pytest.mark.parametrize("face,name", [(0, "trace_xmin"), (1, "trace_xmax"), (2, "trace_ymin"),
                                       (3, "trace_ymax")])
def test_device_trace_kat(gpu_lib, kat, tmp_path, face, name):
    p = _kat_device_params(kat, "ini_slope2", tmp_path)
    x = np.concatenate([kat["trace_q"], kat["trace_dqx"], kat["trace_dqy"]], axis=1)
    out = e2d.eval_device(p, name, x, float(kat["trace_dtdx"]), float(kat["trace_dtdy"]))
    assert np.array_equal(out, kat[f"trace_face{face}"])


@pytest.mark.parametrize("solver", ["hllc", "approx"])
def test_device_riemann_kat(gpu_lib, kat, tmp_path, solver):
    p = _kat_device_params(kat, "ini_slope2", tmp_path)
    x = np.concatenate([kat["riemann_ql"], kat["riemann_qr"]], axis=1)
    out = e2d.eval_device(p, f"riemann_{solver}", x)
    assert np.array_equal(out, kat[f"riemann_{solver}"])


def test_device_hll_vs_oracle(gpu_lib, kat, tmp_path):
    p = _kat_device_params(kat, "ini_slope2", tmp_path)
    x = np.concatenate([kat["riemann_ql"], kat["riemann_qr"]], axis=1)
    out = e2d.eval_device(p, "riemann_hll", x)
    op = po.make_params(**C.oracle_kwargs(str(kat["ini_slope2"])))
    assert np.array_equal(out, po.riemann(op, "hll", kat["riemann_ql"], kat["riemann_qr"]))


def test_device_slopes_edge_values(gpu_lib, tmp_path):
    """Exact integer-pipe limiter on signed zeros, ties, tiny and subnormal
    differences, compared with the oracle's plain FP64 expression."""
    vals = np.array([0.0, -0.0, 1.0, -1.0, 1e-300, -1e-300, 5e-324, -5e-324, 2.2250738585072014e-308,
                     1e-160, -1e-160, 3.0, 0.5, 1.0 + 2 ** -52, 1e300])
    rng = np.random.default_rng(17)
    idx = rng.integers(0, len(vals), size=(3000, 3))
    q5 = np.zeros((3000, 5, 4))
    q5[:, 0, :] = vals[idx[:, 0]][:, None]
    q5[:, 1, :] = vals[idx[:, 1]][:, None]
    q5[:, 2, :] = vals[idx[:, 2]][:, None]
    q5[:, 3, :] = vals[idx[:, 2]][:, None]
    q5[:, 4, :] = vals[idx[:, 1]][:, None]
    for st in (1, 2):
        text = C.ini_text(8, 8, slope_type=st)
        p = e2d.HydroParams.from_ini(C.write_ini(text, str(tmp_path), f"s{st}.ini"))
        out = e2d.eval_device(p, "slopes", q5)
        dqx, dqy = po.slopes(po.make_params(**C.oracle_kwargs(text)), q5)
        np.testing.assert_array_equal(out[:, :4].view(np.int64), dqx.view(np.int64))
        np.testing.assert_array_equal(out[:, 4:].view(np.int64), dqy.view(np.int64))


def test_profiling_mode_same_bits(gpu_lib, runs, tmp_path):
    name = "blast_reflect"
    text = str(runs[f"{name}__ini"])
    with hydro_from_text(text, tmp_path) as h:
        h.set_profiling(True)
        u, dts, t, ns = run_device_loop(h, runs[f"{name}__u0"], 60, 10.0)
        kt = h.kernel_times()
    assert np.array_equal(u, runs[f"{name}__u"])
    assert any(k.startswith("k_step_f64") for k in kt)
    # one prologue per device-loop call, one fused step per step
    assert all(c == (1 if k.endswith("(prologue)") else 60) for k, (_, c) in kt.items())
