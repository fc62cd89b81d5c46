"""The VTK writer (HydroRun::saveVTK, src/HydroRun.h:506-609): the .vti
text of the interior cells in the reference's format, byte for byte.

Golden files (tests/golden/vtk.npz) were written by the reference itself
(oracle/_ref, tests/golden/make_golden.py).  CPU: the reference rewrites the
same bytes, and the library's host-side writer (e2d_write_vtk) produces them
from the same state.  GPU: the state the CUDA path computes, written through
e2d_save_vtk, gives the reference's file -- on a 32x24 implosion and on the
256^2 implosion after 1000 steps (C1, compared by SHA-256)."""
import hashlib
import json
import os

import numpy as np
import pytest

import _cases as C
import euler2d_kokkos_gb300 as e2d

REF_SO = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                      "libe2d_ref.so")


@pytest.fixture(scope="module")
def vtk(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "vtk.npz")))


def small_params(vtk, tmp_path):
    return e2d.HydroParams.from_ini(C.write_ini(str(vtk["small_ini"]), str(tmp_path), "small.ini"))


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="the reference built from its sources is not here")
def test_reference_writes_the_golden_bytes(vtk, tmp_path):
    from oracle.pyoracle import ReferenceLib

    out = tmp_path / "vtk"
    out.mkdir()
    text = str(vtk["small_ini"]) + f"\n[output]\noutputDir={out}\noutputPrefix=ref\n"
    ReferenceLib().save_vtk(C.write_ini(text, str(tmp_path), "ref.ini"), vtk["small_u"], 20)
    assert (out / "ref_0000020.vti").read_bytes() == vtk["small_vti"].tobytes()


def test_host_writer_matches_reference_bytes(vtk, tmp_path):
    p = small_params(vtk, tmp_path)
    u = vtk["small_u"]
    e2d.write_vtk(p, u, str(tmp_path / "left.vti"))
    assert (tmp_path / "left.vti").read_bytes() == vtk["small_vti"].tobytes()
    # the same state in the OpenMP backend's LayoutRight order
    right = np.ascontiguousarray(np.transpose(u, (2, 1, 0)))
    e2d.write_vtk(p, right, str(tmp_path / "right.vti"), layout=e2d.LAYOUT_RIGHT)
    assert (tmp_path / "right.vti").read_bytes() == vtk["small_vti"].tobytes()


def test_host_writer_refuses_bad_arguments(vtk, tmp_path):
    p = small_params(vtk, tmp_path)
    with pytest.raises(ValueError):
        e2d.write_vtk(p, vtk["small_u"][:, :-1], str(tmp_path / "x.vti"))
    with pytest.raises(e2d.E2DError) as ei:
        e2d.write_vtk(p, vtk["small_u"], str(tmp_path / "no_such_dir" / "x.vti"))
    assert ei.value.status == 6  # E2D_EIO


@pytest.mark.gpu
def test_save_vtk_after_device_run_matches_reference(gpu_lib, vtk, tmp_path):
    """20 steps of the device time loop from the reference's own initial
    condition, then saveVTK: the reference's file, byte for byte."""
    with e2d.HydroRun(small_params(vtk, tmp_path)) as h:
        t, ns, _ = h.step_n(20, 10.0, 0.0, 0)
        assert ns == int(vtk["small_nsteps"])
        h.save_vtk(ns % 2, str(tmp_path / "gpu.vti"))
    assert (tmp_path / "gpu.vti").read_bytes() == vtk["small_vti"].tobytes()


@pytest.mark.gpu
def test_save_vtk_of_c1_state_matches_reference(gpu_lib, vtk, golden_dir, tmp_path):
    g = json.load(open(os.path.join(golden_dir, "c1.json")))
    p = e2d.HydroParams.from_ini(C.write_ini(g["ini"], str(tmp_path), "c1.ini"))
    u0 = C.implode_diag_state(256, 256, C.f32(1.4))
    with e2d.HydroRun(p, init_problem=False) as h:
        h.set_state(0, u0)
        h.set_state(1, u0)
        t, ns = 0.0, 0
        while ns < 1000:
            t, ns, _ = h.step_n(1000 - ns, 10.0, t, ns, want_trace=False)
        h.save_vtk(ns % 2, str(tmp_path / "c1.vti"))
    data = (tmp_path / "c1.vti").read_bytes()
    assert len(data) == int(vtk["c1_vti_bytes"])
    assert hashlib.sha256(data).hexdigest() == str(vtk["c1_vti_sha256"])
