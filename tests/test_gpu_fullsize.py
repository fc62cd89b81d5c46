"""The benchmark configurations at their full sizes on the GPU.

- C2, the 4096x4096 blast (FP64, HLLC and HLL): its 200 steps bit for bit
  against the oracle (whose restatement is bit-identical to the reference on
  every golden case), run on the host's cores with OpenMP;
- size-independent properties at 4096^2: mass and energy conservation with
  reflecting walls, and the x <-> y mirror symmetry of the centred blast;
- C3, the 8192x8192 four-quadrant problem: FP32C against the FP64 path after
  20 steps (relative L1 of density <= 1e-5) and the same dt sequence to 1e-6.
"""
import numpy as np
import pytest

import _cases as C
import euler2d_kokkos_gb300 as e2d
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

BLAST_INI = ("[blast]\nradius=0.125\ncenter_x=0.5\ncenter_y=0.5\ndensity_in=1.0\n"
             "density_out=1.0\npressure_in=10.0\npressure_out=0.1\n")


def run(h, nsteps, t_end=10.0):
    t, ns, tr = h.step_n(nsteps, t_end, 0.0, 0)
    assert ns == nsteps
    return h.current(ns), tr


@pytest.mark.parametrize("riemann", ["hllc", "hll"])
def test_c2_blast_4096_bitwise_vs_oracle(gpu_lib, tmp_path, riemann):
    text = C.ini_text(4096, 4096, problem="blast", riemann=riemann, extra=BLAST_INI)
    p = e2d.HydroParams.from_ini(C.write_ini(text, str(tmp_path)))
    with e2d.HydroRun(p) as h:
        u0 = h.U
        u, dts = run(h, 200, C.f32(10.0))
    op = po.make_params(**C.oracle_kwargs(text))
    # the device initialiser (ini reals rounded through float, as ConfigMap does)
    assert np.array_equal(u0, po.init_blast(op, p_out=C.f32(0.1)))
    uo, dto, _, no = po.run(op, u0, 200, C.f32(10.0))
    assert no == 200
    assert np.array_equal(dts, dto)
    assert np.array_equal(u, uo)


def test_c2_blast_4096_conservation_and_symmetry(gpu_lib, tmp_path):
    """Reflecting walls conserve mass and energy (FP64 sums, relative 1e-13
    over 50 steps); the centred blast on a square grid stays mirror-symmetric
    under x <-> y (the x and y updates are added in a fixed order, so the
    mirror is exact only to rounding: 1e-10)."""
    text = C.ini_text(4096, 4096, problem="blast", extra=BLAST_INI)
    p = e2d.HydroParams.from_ini(C.write_ini(text, str(tmp_path)))
    with e2d.HydroRun(p) as h:
        s0 = h.conservation(0)
        t, ns, _ = h.step_n(50, 10.0, 0.0, 0)
        s1 = h.conservation(ns % 2)
        u = h.current(ns)
    for v in (0, 1):
        assert abs(s1[v] - s0[v]) <= 1e-13 * abs(s0[v])
    rho = u[0, 2:-2, 2:-2]
    assert np.max(np.abs(rho - rho.T)) <= 1e-10 * np.max(np.abs(rho))
    mx, my = u[2, 2:-2, 2:-2], u[3, 2:-2, 2:-2]
    assert np.max(np.abs(mx - my.T)) <= 1e-10 * np.max(np.abs(mx))


def test_c3_four_quadrant_8192_fp32c_vs_fp64(gpu_lib):
    kw = dict(problem="four_quadrant", riemann="hllc", gamma0=1.4, cfl=0.8, bc=(2, 2, 2, 2),
              fq_split_x=0.5, fq_split_y=0.5)
    out = {}
    for prec in (e2d.PRECISION_FP64, e2d.PRECISION_FP32C):
        with e2d.HydroRun(e2d.make_params(8192, 8192, precision=prec, **kw)) as h:
            t, ns, tr = h.step_n(20, 10.0, 0.0, 0)
            assert ns == 20
            out[prec] = (h.current(ns)[0, 2:-2, 2:-2].copy(), tr)
    (r64, t64), (r32, t32) = out[e2d.PRECISION_FP64], out[e2d.PRECISION_FP32C]
    assert np.max(np.abs(t32 - t64) / t64) < 1e-6
    assert np.abs(r32 - r64).sum() / np.abs(r64).sum() < 1e-5
