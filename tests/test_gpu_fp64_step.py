"""The fused FP64 step of the device time loop (k_step_f64: one launch per
step, TMA-staged tiles, the next step's CFL maximum folded in the epilogue)
against the two-launch step and the oracle, bit for bit.

Grids are chosen so that every staging path runs: tiles whose 2-cell halo
box is interior (one TMA copy), tiles whose halo reaches ghost cells
(gathered through the boundary map), and grids with an odd row length
(isize odd: no tensor map can be encoded, every tile is gathered)."""
import os

import numpy as np
import pytest

import _cases as C
import euler2d_kokkos_gb300 as e2d
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

G14 = C.f32(1.4)
# (nx, ny, boundary types): isize even with interior tiles; isize odd;
# periodic; mixed
GRIDS = [(200, 130, (1, 1, 1, 1)), (157, 96, (2, 2, 2, 2)), (160, 160, (3, 3, 3, 3)), (222, 140, (1, 2, 3, 3))]


def params(nx, ny, bc, riemann="hllc"):
    return e2d.make_params(nx, ny, problem="implode", riemann=riemann, gamma0=1.4, cfl=0.8, slope_type=2.0, bc=bc)


def run_loop(p, u0, steps, chunk, env, monkeypatch):
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    try:
        with e2d.HydroRun(p, init_problem=False) as h:
            h.set_state(0, u0)
            h.set_state(1, u0)
            t, ns, tr = 0.0, 0, []
            while ns < steps:
                t, ns, d = h.step_n(min(chunk, steps - ns), 10.0, t, ns)
                tr.append(d)
            return h.get_state(0), h.get_state(1), np.concatenate(tr), t
    finally:
        for k in env:
            monkeypatch.delenv(k)


@pytest.mark.parametrize("nx,ny,bc", GRIDS)
def test_fused_step_matches_oracle(gpu_lib, monkeypatch, nx, ny, bc):
    """Both states (ghosts included), every dt and t after 30 steps equal the
    oracle's, which reproduces the reference bit for bit."""
    u0 = C.smooth_state(nx, ny, G14, seed=nx + ny)
    u_a, u_b, tr, t = run_loop(params(nx, ny, bc), u0, 30, 11, {}, monkeypatch)
    op = po.make_params(nx, ny, gamma0=1.4, cfl=0.8, slope_type=2.0, bc=bc, riemann="hllc")
    uo, dto, to, no = po.run(op, u0, 30, 10.0)
    assert no == 30 and t == to
    assert np.array_equal(tr, dto)
    assert np.array_equal(u_a, uo)  # 30 steps: the result is in U


@pytest.mark.parametrize("tile", ["0", "1", "2", "3"])
@pytest.mark.parametrize("riemann", ["hllc", "hll", "approx"])
def test_fused_step_equals_two_launch_step(gpu_lib, monkeypatch, tile, riemann):
    """Every tile shape and solver: the fused step's two states and dt
    sequence equal those of the two-launch step (E2D_F64_SPLIT=1)."""
    for nx, ny, bc in GRIDS[:2]:
        p = params(nx, ny, bc, riemann)
        u0 = C.smooth_state(nx, ny, G14, seed=3 * nx + ny)
        fused = run_loop(p, u0, 17, 17, {"E2D_F64_TILE": tile}, monkeypatch)
        split = run_loop(p, u0, 17, 17, {"E2D_F64_TILE": tile, "E2D_F64_SPLIT": "1"}, monkeypatch)
        for a, b in zip(fused, split):
            assert np.array_equal(a, b), (nx, ny, tile, riemann)


def test_fused_step_stops_at_t_end_and_resumes(gpu_lib, monkeypatch):
    """The dt clamp at t_end, the no-op steps after it inside one call, and a
    second call resuming from the returned (t, nstep): as one oracle run."""
    nx, ny, bc = GRIDS[0]
    p = params(nx, ny, bc)
    u0 = C.implode_diag_state(nx, ny, G14)
    with e2d.HydroRun(p, init_problem=False) as h:
        h.set_state(0, u0)
        h.set_state(1, u0)
        t, ns, tr1 = h.step_n(5, 0.01, 0.0, 0)
        t, ns, tr2 = h.step_n(64, 0.01, t, ns)  # t_end reached inside the call
        u = h.current(ns)
    op = po.make_params(nx, ny, gamma0=1.4, cfl=0.8, slope_type=2.0, bc=bc, riemann="hllc")
    uo, dto, to, no = po.run(op, u0, 1000, 0.01)
    assert ns == no and t == to
    assert np.array_equal(np.concatenate([tr1, tr2]), dto)
    assert np.array_equal(u, uo)


def test_fused_step_wait_runs_out_with_etimeout(gpu_lib, monkeypatch):
    """Failure detection without a GPU fault: with E2D_TEST_WAIT_TIMEOUT=1,
    tile (1, 1) of the fused step never issues its TMA copy, so its bounded
    mbarrier wait gives up after 1 s, waits (bounded) once more and flags the
    step; step_n returns E2D_ETIMEOUT and the context stays usable."""
    p = params(256, 256, (1, 1, 1, 1))
    u0 = C.implode_diag_state(256, 256, G14)
    monkeypatch.setenv("E2D_TEST_WAIT_TIMEOUT", "1")
    with e2d.HydroRun(p, init_problem=False) as h:
        h.set_state(0, u0)
        with pytest.raises(e2d.E2DError) as ei:
            h.step_n(1, 10.0, 0.0, 0)
        assert ei.value.status == 4  # E2D_ETIMEOUT
    monkeypatch.delenv("E2D_TEST_WAIT_TIMEOUT")
    with e2d.HydroRun(p, init_problem=False) as h:
        h.set_state(0, u0)
        h.set_state(1, u0)
        t, ns, _ = h.step_n(2, 10.0, 0.0, 0)
        assert ns == 2 and np.isfinite(h.current(ns)).all()


def test_fast_forms_do_not_depend_on_the_tile_shape(gpu_lib, monkeypatch):
    """The fast forms (not bit-identical to the reference) still give one
    result whatever the tile: 32 x 16 (default) and 32 x 32 agree bit for bit."""
    nx, ny, bc = GRIDS[0]
    p = params(nx, ny, bc)
    p.precision = e2d.PRECISION_FP64_FAST
    p.init()
    u0 = C.smooth_state(nx, ny, G14, seed=5)
    a = run_loop(p, u0, 15, 15, {"E2D_F64_TILE": "0"}, monkeypatch)
    b = run_loop(p, u0, 15, 15, {"E2D_F64_TILE": "1"}, monkeypatch)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_device_loop_cache_follows_state_changes(gpu_lib):
    """A device-loop call reuses the primitives and CFL maximum the previous
    call left on the device only while nothing has changed the state: after
    set_state, godunov_unsplit or make_boundaries between calls, the result
    is that of a fresh handle run from the changed state."""
    nx, ny, bc = GRIDS[0]
    p = params(nx, ny, bc)
    ua = C.smooth_state(nx, ny, G14, seed=21)
    ub = C.smooth_state(nx, ny, G14, seed=22)

    def fresh(u0, steps):
        with e2d.HydroRun(p, init_problem=False) as f:
            f.set_state(0, u0)
            f.set_state(1, u0)
            t, ns, tr = f.step_n(steps, 10.0, 0.0, 0)
            return f.current(ns), tr

    with e2d.HydroRun(p, init_problem=False) as h:
        h.set_state(0, ua)
        h.set_state(1, ua)
        h.step_n(4, 10.0, 0.0, 0)          # leaves U's primitives cached
        h.set_state(0, ub)                 # ... which set_state must drop
        h.set_state(1, ub)
        t, ns, tr = h.step_n(6, 10.0, 0.0, 0)
        u, d = fresh(ub, 6)
        assert np.array_equal(h.current(ns), u) and np.array_equal(tr, d)
        # a host-driven step between two device-loop calls
        dt = h.compute_dt(ns % 2)
        h.godunov_unsplit(ns, dt)
        t2, ns2, tr2 = h.step_n(3, 10.0, t + dt, ns + 1)
        with e2d.HydroRun(p, init_problem=False) as f:
            f.set_state(0, ub)
            f.set_state(1, ub)
            tf, nf, _ = f.step_n(6, 10.0, 0.0, 0)
            f.godunov_unsplit(nf, f.compute_dt(nf % 2))
            tf, nf, trf = f.step_n(3, 10.0, tf + dt, nf + 1)
            assert np.array_equal(h.current(ns2), f.current(nf)) and np.array_equal(tr2, trf)
