"""The opt-in fast FP64 step (precision fp64_fast: FMAs and one
Newton-refined reciprocal per denominator in place of divisions; not
bit-identical) held to the reference's stated tolerance: every dt within
1e-12 relative and every variable within 1e-10 relative L1 of the bit-exact
FP64 path -- itself bit-identical to the reference -- on the implosion
(256^2, 1000 steps: the 1000 dts are also compared with the reference's
golden ones) and on the 4096^2 blast (200 steps, HLLC and HLL)."""
import json
import os

import numpy as np
import pytest

import _cases as C
import euler2d_kokkos_gb300 as e2d

pytestmark = pytest.mark.gpu

DT_TOL = 1e-12
L1_TOL = 1e-10


def rel_l1(a, b):
    a, b = a[:, 2:-2, 2:-2], b[:, 2:-2, 2:-2]
    return max(float(np.abs(a[v] - b[v]).sum() / np.abs(b[v]).sum()) for v in range(4))


def run(p, u0, steps, t_end=10.0):
    with e2d.HydroRun(p, init_problem=u0 is None) as h:
        if u0 is not None:
            h.set_state(0, u0)
            h.set_state(1, u0)
        t, ns, tr = 0.0, 0, []
        while ns < steps and t < t_end:
            t, ns, d = h.step_n(min(256, steps - ns), t_end, t, ns)
            tr.append(d)
        return h.current(ns), np.concatenate(tr), ns


def fast_copy(p):
    q = p.copy()
    q.precision = e2d.PRECISION_FP64_FAST
    return q.init()


def test_fast_c1_implode_within_tolerance(gpu_lib, golden_dir, tmp_path):
    g = json.load(open(os.path.join(golden_dir, "c1.json")))
    p = e2d.HydroParams.from_ini(C.write_ini(g["ini"], str(tmp_path), "c1.ini"))
    u0 = C.implode_diag_state(256, 256, C.f32(1.4))
    ue, dte, _ = run(p, u0, 1000)
    uf, dtf, nf = run(fast_copy(p), u0, 1000)
    ref_dt = np.array([float.fromhex(x) for x in g["dt_hex"]])
    assert nf == 1000 and np.array_equal(dte, ref_dt)
    assert np.max(np.abs(dtf - ref_dt) / ref_dt) < DT_TOL
    assert rel_l1(uf, ue) < L1_TOL


@pytest.mark.parametrize("riemann", ["hllc", "hll"])
def test_fast_c2_blast_within_tolerance(gpu_lib, riemann):
    p = e2d.make_params(4096, 4096, problem="blast", riemann=riemann, gamma0=1.4, cfl=0.8, slope_type=2.0,
                        bc=(1, 1, 1, 1), blast_radius=0.125, blast_center_x=0.5, blast_center_y=0.5,
                        blast_density_in=1.0, blast_density_out=1.0, blast_pressure_in=10.0,
                        blast_pressure_out=0.1)
    ue, dte, _ = run(p, None, 200)
    uf, dtf, nf = run(fast_copy(p), None, 200)
    assert nf == 200
    assert np.max(np.abs(dtf - dte) / dte) < DT_TOL
    assert rel_l1(uf, ue) < L1_TOL


def test_fast_is_refused_where_it_does_not_run(gpu_lib):
    p = fast_copy(e2d.make_params(64, 64, problem="implode", riemann="hllc", gamma0=1.4, cfl=0.8))
    with e2d.HydroRun(p) as h:
        with pytest.raises(e2d.E2DError) as ei:
            h.godunov_unsplit(0, 1e-4)
        assert ei.value.status == 1
    with e2d.Batch(pool_bytes=64 << 20) as b:
        with pytest.raises(e2d.E2DError) as ei:
            b.admit(p, 0.01)
        assert ei.value.status == 1
    q = p.copy()
    q.implementationVersion = 1
    with pytest.raises(e2d.E2DError) as ei:
        e2d.HydroRun(q.init())
    assert ei.value.status == 1
