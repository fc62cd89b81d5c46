"""The Sedov post-processing (src/main.cpp:175-179): the radial density
profile of ComputeRadialProfileFunctor (src/ComputeRadialProfileFunctor.h)
and its .npy output (src/cnpy/cnpy.h).  CPU: the oracle's restatement and
the library's .npy writer against the files the reference itself wrote
(tests/golden/sedov.npz).  GPU: the device profile through the C ABI and the
command-line driver's output files."""
import hashlib
import io
import os
import subprocess

import numpy as np
import pytest

import _cases as C
import euler2d_kokkos_gb300 as e2d
from oracle import pyoracle as O


@pytest.fixture(scope="module")
def sedov(golden_dir):
    z = dict(np.load(os.path.join(golden_dir, "sedov.npz")))
    for nb in C.SEDOV_NBINS:
        z[f"dist_{nb}"] = np.load(io.BytesIO(z[f"dist_npy_{nb}"].tobytes()))
        z[f"prof_{nb}"] = np.load(io.BytesIO(z[f"prof_npy_{nb}"].tobytes()))
    return z


def golden_state(z):
    """A state whose density plane is the reference's after 60 steps (the
    profile reads only rho)."""
    u = np.zeros((4,) + z["rho"].shape)
    u[0] = z["rho"]
    return u


def sum_bound(prof_ref, counts):
    """Rigorous bound between two FP64 means of the same positive values
    summed in different orders: (n - 1) u sum|x| for the sum, plus the
    division's rounding, relative to the mean."""
    u = 2.0 ** -53
    return (counts + 2) * u * np.abs(prof_ref)


@pytest.mark.parametrize("nbins", C.SEDOV_NBINS)
def test_oracle_profile_is_the_reference(sedov, nbins):
    p = O.make_params(**C.oracle_kwargs(C.sedov_ini(nbins)))
    d, prof, cnt = O.radial_profile(p, golden_state(sedov), nbins)
    assert np.array_equal(d, sedov[f"dist_{nbins}"])
    assert np.array_equal(prof, sedov[f"prof_{nbins}"], equal_nan=True)
    # empty rings are 0/0 in both
    assert np.array_equal(np.isnan(prof), cnt == 0)


def test_profile_counts_every_cell_once(sedov):
    """Every cell whose ring index is < nbins is counted once; the ghost
    corners (ring index >= nbins) are the only cells left out."""
    p = O.make_params(**C.oracle_kwargs(C.sedov_ini(40)))
    _, _, cnt = O.radial_profile(p, golden_state(sedov), 40)
    assert 0 < (68 * 68 - cnt.sum()) < 4 * 2 * 2 * 4


@pytest.mark.parametrize("nbins", C.SEDOV_NBINS)
def test_save_npy_bytes_equal_reference_files(sedov, tmp_path, nbins):
    for kind in ("dist", "prof"):
        f = tmp_path / f"{kind}.npy"
        e2d.save_npy(str(f), sedov[f"{kind}_{nbins}"])
        assert f.read_bytes() == sedov[f"{kind}_npy_{nbins}"].tobytes()


@pytest.mark.gpu
def test_device_profile_of_the_reference_run(gpu_lib, sedov, tmp_path):
    """The reference's initial condition and 60 steps on the FP64 path (bit
    for bit), then the device profile: distances and counts exact, means
    within the summation-order bound of the reference's serial sums."""
    params = e2d.HydroParams.from_ini(C.write_ini(C.sedov_ini(40), str(tmp_path)))
    with e2d.HydroRun(params) as h:
        t, ns, dts = h.step_n(60, params.tEnd, 0.0, 0)
        assert ns == int(sedov["nsteps"]) and np.array_equal(dts, sedov["dt"])
        u = h.current(ns)
        assert hashlib.sha256(np.ascontiguousarray(u).tobytes()).digest() == sedov["sha256_state"].tobytes()
        p = O.make_params(**C.oracle_kwargs(C.sedov_ini(40)))
        for nb in C.SEDOV_NBINS:
            d, prof, cnt = h.radial_profile(0, nb)
            _, _, cnt_o = O.radial_profile(p, u, nb)
            ref = sedov[f"prof_{nb}"]
            assert np.array_equal(d, sedov[f"dist_{nb}"])
            assert np.array_equal(cnt, cnt_o)
            assert np.array_equal(np.isnan(prof), np.isnan(ref))
            ok = ~np.isnan(ref)
            assert np.all(np.abs(prof[ok] - ref[ok]) <= sum_bound(ref[ok], cnt[ok]))
        # the [blast] nbins key is the default ring count
        d, prof, _ = h.radial_profile()
        assert len(d) == 40


@pytest.mark.gpu
def test_device_profile_fp32c_and_errors(gpu_lib, sedov, tmp_path):
    params = e2d.HydroParams.from_ini(C.write_ini(C.sedov_ini(40), str(tmp_path)))
    params.precision = e2d.PRECISION_FP32C
    with e2d.HydroRun(params) as h:
        t, ns, _ = h.step_n(60, params.tEnd, 0.0, 0)
        _, prof, _ = h.radial_profile(ns % 2, 40)
        ref = sedov["prof_40"]
        assert np.max(np.abs(prof - ref) / ref) < 1e-5
        bad = h.current(ns)
        bad[0, 30, 30] = np.nan
        h.set_state(0, bad)
        with pytest.raises(e2d.E2DError) as ei:
            h.radial_profile(0, 40)
        assert ei.value.status == 3  # E2D_ENUMERIC


@pytest.mark.gpu
def test_cli_writes_sedov_npy_files(gpu_lib, sedov, tmp_path):
    """euler2d_gb300 on the ini: the two .npy files of src/main.cpp:175-179."""
    ini = C.write_ini(C.sedov_ini(40), str(tmp_path))
    exe = os.path.join(os.path.dirname(e2d.__file__), "_build", "euler2d_gb300")
    r = subprocess.run([exe, ini], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    dist = (tmp_path / "sedov_blast_radial_distances.npy").read_bytes()
    assert dist == sedov["dist_npy_40"].tobytes()
    prof = np.load(tmp_path / "sedov_blast_density_profile.npy")
    ref = sedov["prof_40"]
    _, _, cnt = O.radial_profile(O.make_params(**C.oracle_kwargs(C.sedov_ini(40))), golden_state(sedov), 40)
    assert np.all(np.abs(prof - ref) <= sum_bound(ref, cnt))
