"""e2d_godunov_unsplit_noalloc: one FP64 step on caller-owned device buffers
with no allocation by the library (its scratch is a fixed file-scope device
array).  It serves callers that cannot let a library call cudaMalloc -- hosts
with their own fixed device pool, latency-critical loops that cannot take
cudaMalloc's implicit synchronisation, code that keeps no handle.

Checked here through the C ABI against the handle-based e2d_godunov_unsplit:
two calls in a row (U -> U2 -> U), tolerance 0 (the FP64 path is bit-exact).
This file is collected last so that a run stopping at its first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

import _cases as C
import euler2d_kokkos_gb300 as e2d

pytestmark = pytest.mark.gpu


def _params(tmp_path, nx, ny, bc=(1, 2, 3, 3)):
    text = C.ini_text(nx, ny, bc=bc)
    return e2d.HydroParams.from_ini(C.write_ini(text, str(tmp_path)))


def test_noalloc_two_calls_match_handle_entry_point(gpu_lib, tmp_path):
    import torch

    nx, ny = 120, 90
    p = _params(tmp_path, nx, ny)
    u0 = C.smooth_state(nx, ny, C.f32(1.4), seed=31)
    with e2d.HydroRun(p, init_problem=False) as h:
        h.set_state(0, u0)
        h.set_state(1, u0)
        dt1 = h.compute_dt(0)
        h.godunov_unsplit(0, dt1)
        dt2 = h.compute_dt(1)
        h.godunov_unsplit(1, dt2)
        want_u, want_u2 = h.U, h.U2

    a = torch.from_numpy(u0.copy()).cuda()
    b = torch.zeros_like(a)
    L = gpu_lib
    stream = torch.cuda.current_stream().cuda_stream
    assert L.e2d_godunov_unsplit_noalloc(ctypes.byref(p._raw), a.data_ptr(), b.data_ptr(), dt1, stream) == 0
    assert L.e2d_godunov_unsplit_noalloc(ctypes.byref(p._raw), b.data_ptr(), a.data_ptr(), dt2, stream) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(a.cpu().numpy(), want_u)
    np.testing.assert_array_equal(b.cpu().numpy(), want_u2)


def test_noalloc_refuses_grids_above_its_scratch(gpu_lib, tmp_path):
    """A grid above E2D_NOALLOC_MAX_CELLS cells is refused before any launch."""
    import torch

    p = _params(tmp_path, 520, 520)
    assert p.isize * p.jsize > (1 << 18)
    a = torch.zeros(4 * p.isize * p.jsize, dtype=torch.float64, device="cuda")
    b = torch.zeros_like(a)
    rc = gpu_lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p._raw), a.data_ptr(), b.data_ptr(), 1e-3, None)
    assert rc == 1  # E2D_EINVAL
    torch.cuda.synchronize()
    assert float(b.abs().sum()) == 0.0  # nothing was written
