"""The C++ mirror of the reference's driver API (include/euler2d_gb300.hpp:
ConfigMap, HydroParams, HydroRun) linked and run: tests/mirror_driver.cpp is
src/main.cpp's loop (76-145) written against it.  CPU: it compiles and links
against libe2d_gb300.so.  GPU: run on golden inis, its dt sequence, final
state and .vti output equal the reference's bit for bit / byte for byte."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

import _cases as C
import euler2d_kokkos_gb300 as e2d

TESTS = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(TESTS)
# the golden runs that start from the reference's own initial condition
REF_IC_CASES = ["implode_ref_ini", "blast_reflect", "four_quadrant_absorb", "discontinuity_absorb",
                "shocked_bubble"]


def build_driver(out_dir):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    lib = e2d.load_library()._name
    libdir = os.path.dirname(lib)
    exe = os.path.join(str(out_dir), "mirror_driver")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(TESTS, "mirror_driver.cpp"), "-o", exe, "-L", libdir, "-le2d_gb300",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run_driver(exe, text, tmp_path, name, limit):
    out = tmp_path / f"vti_{name}"
    out.mkdir()
    ini = C.write_ini(text + f"\n[output]\noutputDir={out}\noutputPrefix=mirror\n", str(tmp_path), f"{name}.ini")
    res = tmp_path / f"{name}.bin"
    r = subprocess.run([exe, ini, str(limit), str(res)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = res.read_bytes()
    ns = struct.unpack_from("<i", raw, 0)[0]
    t = struct.unpack_from("<d", raw, 4)[0]
    dts = np.frombuffer(raw, dtype=np.float64, count=ns, offset=12)
    u = np.frombuffer(raw, dtype=np.float64, offset=12 + 8 * ns)
    return ns, t, dts, u, out


def test_mirror_driver_compiles_and_links(tmp_path):
    assert os.access(build_driver(tmp_path), os.X_OK)


@pytest.mark.gpu
def test_mirror_driver_matches_reference_bitwise(gpu_lib, runs, tmp_path):
    exe = build_driver(tmp_path)
    for name in REF_IC_CASES:
        text = str(runs[f"{name}__ini"])
        ns, t, dts, u, _ = run_driver(exe, text, tmp_path, name, C.run_cases()[name]["nsteps"])
        assert ns == int(runs[f"{name}__nsteps"]), name
        assert np.array_equal(dts, runs[f"{name}__dt"]), name
        assert t == float(runs[f"{name}__t"]), name
        assert np.array_equal(u.reshape(runs[f"{name}__u"].shape), runs[f"{name}__u"]), name


@pytest.mark.gpu
def test_mirror_driver_writes_the_reference_vti(gpu_lib, golden_dir, tmp_path):
    vtk = np.load(os.path.join(golden_dir, "vtk.npz"))
    exe = build_driver(tmp_path)
    ns, _, _, _, out = run_driver(exe, str(vtk["small_ini"]), tmp_path, "small", 20)
    assert ns == int(vtk["small_nsteps"])
    assert (out / f"mirror_{ns:07d}.vti").read_bytes() == vtk["small_vti"].tobytes()
