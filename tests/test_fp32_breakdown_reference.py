"""The FP32 breakdown of the FP32C regression flow (_cases.BREAKDOWN_*) is
the reference's too: its own solver built in single precision
(oracle/_ref/libe2d_ref32.so, the reference's sources without USE_DOUBLE)
turns non-finite on that flow by step 480, near the vertical split, while
its FP64 build (libe2d_ref.so) stays finite.  CPU only; needs the reference
builds, made where the reference tree is present."""
import os

import numpy as np
import pytest

import _cases as C
from euler2d_kokkos_gb300 import workloads as W
from oracle import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF32_SO = os.path.join(ROOT, "oracle", "_ref", "libe2d_ref32.so")
STEPS = 480  # the float build turns non-finite between steps 440 and 480


def test_reference_single_precision_build_breaks_down_where_fp64_does_not(tmp_path):
    if not (os.path.exists(REF32_SO) and os.path.exists(po.REF_SO)):
        pytest.skip("the reference builds are made only where the reference tree is present")
    nx, ny = C.BREAKDOWN_NX, C.BREAKDOWN_NY
    text = C.ini_text(nx, ny, bc=(2, 2, 2, 2), problem="four_quadrant", riemann="hllc", gamma0=1.4,
                      cfl=0.8, tEnd=repr(C.BREAKDOWN_T_END), nStepmax=100000)
    ini = C.write_ini(text, str(tmp_path), "breakdown.ini")
    u0 = W.four_quadrant_state(nx, ny, C.BREAKDOWN_STATES, gamma=C.f32(1.4), split=(0.5, 0.5))
    u32, _, _, n32 = po.ReferenceLib(REF32_SO).run(ini, u0, STEPS)
    u64, _, _, n64 = po.ReferenceLib().run(ini, u0, STEPS)
    assert n32 == n64 == STEPS
    bad = ~np.isfinite(u32[0])
    assert bad.any()
    cols = np.nonzero(bad.any(axis=0))[0] - 2  # interior column index
    assert abs(np.median(cols) - nx // 2) < 0.1 * nx
    assert np.isfinite(u64).all() and u64[0, 2:-2, 2:-2].min() > 0
