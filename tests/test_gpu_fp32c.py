"""The FP32 path with compensated (hi, lo) update against the FP64 path.

Tolerances (relative L1 of density over the interior, FP64 accumulation):
FP32C_L1_TOL below.  The FP64 path is itself bit-identical to the reference
(test_gpu_parity.py), so it is the oracle here."""
import numpy as np
import pytest

import _cases as C
import euler2d_kokkos_gb300 as e2d

pytestmark = pytest.mark.gpu

FP32C_L1_TOL = 1e-5


def pair(text, tmp_path, u0=None, riemann=None):
    p64 = e2d.HydroParams.from_ini(C.write_ini(text, str(tmp_path), "a.ini"))
    if riemann:
        p64.riemannSolverType = e2d.RIEMANN[riemann]
    p32 = p64.copy()
    p32.precision = e2d.PRECISION_FP32C
    h64 = e2d.HydroRun(p64.init())
    h32 = e2d.HydroRun(p32.init())
    if u0 is not None:
        for h in (h64, h32):
            h.set_state(0, u0)
            h.set_state(1, u0)
    return h64, h32


def rel_l1(h32, w32, h64, w64, var=0):
    d, r = h32.l1_diff(w32, h64, w64, var)
    return d / r


@pytest.mark.parametrize("case,nsteps", [("implode_diag", 100), ("blast_reflect", 60),
                                         ("four_quadrant_absorb", 60), ("periodic_smooth", 50),
                                         ("mixed_bc_smooth", 40)])
def test_fp32c_close_to_fp64(gpu_lib, runs, tmp_path, case, nsteps):
    text = str(runs[f"{case}__ini"])
    h64, h32 = pair(text, tmp_path, runs[f"{case}__u0"])
    t64, n64, dt64 = h64.step_n(nsteps, 10.0, 0.0, 0)
    t32, n32, dt32 = h32.step_n(nsteps, 10.0, 0.0, 0)
    assert n64 == n32 == nsteps
    assert np.allclose(dt32, dt64, rtol=1e-5, atol=0)
    # fixed-time comparison: both runs end at nearly the same time
    err = rel_l1(h32, n32 % 2, h64, n64 % 2)
    assert err < FP32C_L1_TOL, err
    # the FP64 path matches the reference bit for bit
    assert np.array_equal(h64.current(n64), runs[f"{case}__u"])


def test_fp32c_initial_conditions_equal_fp64(gpu_lib, tmp_path):
    text = C.ini_text(64, 48, problem="four_quadrant", bc=(2, 2, 2, 2))
    h64, h32 = pair(text, tmp_path)
    u64, u32 = h64.U, h32.U
    # hi + lo represents every FP64 initial value to ~2^-48 relative
    assert np.allclose(u32, u64, rtol=2e-14, atol=0)


def test_fp32c_mass_conserved_periodic(gpu_lib, tmp_path):
    """Every face flux is added to one cell and subtracted from its neighbour
    with compensated sums: total mass/momentum/energy drift stays at FP64
    round-off level on a periodic domain."""
    text = C.ini_text(96, 80, bc=(3, 3, 3, 3))
    u0 = C.smooth_state(96, 80, C.f32(1.4), seed=21)
    _, h32 = pair(text, tmp_path, u0)
    s0 = h32.conservation(0)
    t, ns, _ = h32.step_n(200, 10.0, 0.0, 0)
    s1 = h32.conservation(ns % 2)
    rel = np.abs(s1 - s0) / np.abs(s0).clip(1e-300)
    assert rel[0] < 1e-10 and rel[1] < 1e-10, rel


@pytest.mark.parametrize("riemann", ["hll", "approx"])
def test_fp32c_other_solvers(gpu_lib, runs, tmp_path, riemann):
    case = "four_quadrant_absorb"
    text = str(runs[f"{case}__ini"]).replace("riemann=hllc", f"riemann={riemann}")
    h64, h32 = pair(text, tmp_path, runs[f"{case}__u0"])
    _, n64, _ = h64.step_n(30, 10.0, 0.0, 0)
    _, n32, _ = h32.step_n(30, 10.0, 0.0, 0)
    assert rel_l1(h32, n32 % 2, h64, n64 % 2) < FP32C_L1_TOL


def test_fp32c_host_loop_matches_device_loop(gpu_lib, runs, tmp_path):
    case = "blast_reflect"
    text = str(runs[f"{case}__ini"])
    _, ha = pair(text, tmp_path, runs[f"{case}__u0"])
    _, hb = pair(text, tmp_path, runs[f"{case}__u0"])
    t, ns, dts = ha.step_n(40, 10.0, 0.0, 0)
    tb, nb = 0.0, 0
    for _ in range(40):
        dt = hb.compute_dt(nb % 2)
        hb.godunov_unsplit(nb, dt)
        nb += 1
        tb += dt
    assert abs(tb - t) <= 1e-6 * t
    assert rel_l1(hb, nb % 2, ha, ns % 2) < 1e-5


def test_fp32c_conservation_audit_fp64_matches_numpy(gpu_lib, tmp_path):
    text = C.ini_text(40, 30)
    u0 = C.smooth_state(40, 30, C.f32(1.4), seed=5)
    h64, _ = pair(text, tmp_path, u0)
    s = h64.conservation(0)
    inner = u0[:, 2:-2, 2:-2].reshape(4, -1)
    ref = inner.sum(axis=1)
    # summation order differs from numpy's: bound by the sum of magnitudes
    assert np.all(np.abs(s - ref) <= 1e-13 * np.abs(inner).sum(axis=1)), (s, ref)


@pytest.mark.parametrize("nx,ny,bc", [(2, 2, (1, 1, 1, 1)), (3, 5, (2, 2, 2, 2)), (7, 121, (3, 3, 1, 2)),
                                      (59, 17, (1, 2, 3, 3)), (60, 16, (3, 3, 3, 3)),
                                      (61, 33, (2, 1, 1, 2)), (121, 7, (1, 1, 2, 2)),
                                      (122, 48, (3, 3, 2, 2))])
def test_fp32c_edge_sizes(gpu_lib, tmp_path, nx, ny, bc):
    """Grids narrower than a 60-column strip, with 1- or 2-column
    remainders, shorter than a 16-row fold unit, and every boundary type on
    the strips that read ghost columns and rows through the boundary map:
    FP32C stays within the tolerance of FP64 and dt agrees to 1e-5."""
    g14 = C.f32(1.4)
    text = C.ini_text(nx, ny, bc=bc)
    u0 = C.smooth_state(nx, ny, g14, seed=nx * 1000 + ny)
    h64, h32 = pair(text, tmp_path, u0)
    t64, n64, dt64 = h64.step_n(20, 10.0, 0.0, 0)
    t32, n32, dt32 = h32.step_n(20, 10.0, 0.0, 0)
    assert n64 == n32 == 20
    assert np.allclose(dt32, dt64, rtol=1e-5, atol=0)
    assert rel_l1(h32, n32 % 2, h64, n64 % 2) < FP32C_L1_TOL


def test_fp32c_nonfinite_state_reports_enumeric(gpu_lib, tmp_path):
    """A NaN in the state stops the FP32C device loop with E2D_ENUMERIC, as
    on the FP64 path."""
    text = C.ini_text(64, 48, problem="implode")
    _, h32 = pair(text, tmp_path)
    u = h32.U
    u[0, 20, 20] = np.nan
    h32.set_state(0, u)
    with pytest.raises(e2d.E2DError) as ei:
        h32.step_n(10, 10.0, 0.0, 0)
    assert ei.value.status == 3  # E2D_ENUMERIC


TMA_VARIANT = 6  # rows staged by TMA, waits on mbarriers


@pytest.mark.parametrize("variant", [str(TMA_VARIANT), "7"])
@pytest.mark.parametrize("strip_h", ["16", "64"])
def test_tma_variant_matches_default(gpu_lib, monkeypatch, variant, strip_h):
    """The TMA-staged variants -- one row per copy (6) and two rows per copy
    (7) -- give the same bits as the default (cp.async) variant on a grid
    with interior, boundary and ghost-row strips."""
    p = e2d.make_params(300, 200, problem="implode", riemann="hllc", gamma0=1.4, cfl=0.8,
                        implode_shape=1, bc=(1, 3, 2, 1), precision=e2d.PRECISION_FP32C)
    monkeypatch.setenv("E2D_F32C_STRIP_H", strip_h)
    out = []
    for v in ("4", variant):
        monkeypatch.setenv("E2D_F32C_VARIANT", v)
        with e2d.HydroRun(p) as h:
            _, ns, trace = h.step_n(30, 10.0, 0.0, 0)
            out.append((h.current(ns), trace))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_row_staging_wait_runs_out_with_etimeout(gpu_lib, monkeypatch):
    """Failure detection without a GPU fault: with E2D_TEST_WAIT_TIMEOUT=1 the
    TMA variant never stages the first row of strip (1, 0), so that warp's
    bounded mbarrier wait gives up after its 1 s limit, drains its copies in
    flight and flags the step.  step_n returns E2D_ETIMEOUT, a batch stops
    the solve (query E2D_ETIMEOUT), and the context stays usable: the same
    step runs normally once the switch is off."""
    p = e2d.make_params(256, 256, problem="implode", riemann="hllc", gamma0=1.4, cfl=0.8,
                        implode_shape=1, precision=e2d.PRECISION_FP32C)
    monkeypatch.setenv("E2D_TEST_WAIT_TIMEOUT", "1")
    monkeypatch.setenv("E2D_F32C_VARIANT", str(TMA_VARIANT))
    with e2d.HydroRun(p) as h:
        with pytest.raises(e2d.E2DError) as ei:
            h.step_n(1, 10.0, 0.0, 0)
        assert ei.value.status == 4  # E2D_ETIMEOUT
    with e2d.Batch(pool_bytes=64 << 20) as b:
        b.set_tuning(TMA_VARIANT, [64, 64, 64])
        i = b.admit(p, 0.01)
        b.run(1)
        with pytest.raises(e2d.E2DError) as ei:
            b.query(i)
        assert ei.value.status == 4
        _, _, active, ok = b.poll(i)
        assert not active and not ok
    monkeypatch.delenv("E2D_TEST_WAIT_TIMEOUT")
    with e2d.HydroRun(p) as h:  # still the TMA variant
        t, ns, _ = h.step_n(2, 10.0, 0.0, 0)
        assert ns == 2 and np.isfinite(h.current(ns)).all()
