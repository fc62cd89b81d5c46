"""Shared definitions of the parity cases: ini texts in the reference's
format and seeded initial states.  Used by tests/golden/make_golden.py (which
runs the reference on them) and by the tests (which run the oracle and the
GPU path on the same inputs)."""
from __future__ import annotations

import os
import tempfile

import numpy as np


def ini_text(nx, ny, *, bc=(1, 1, 1, 1), problem="implode", riemann="hllc", gamma0=1.4,
             cfl=0.8, slope_type=2, tEnd=10.0, nStepmax=100, xmin=0.0, xmax=1.0, ymin=0.0,
             ymax=1.0, extra: str = "") -> str:
    """An ini file in the layout of the reference's src/test_*.ini files."""
    return f"""[run]
tEnd={tEnd}
nStepmax={nStepmax}
nOutput=-1

[mesh]
nx={nx}
ny={ny}
xmin={xmin}
xmax={xmax}
ymin={ymin}
ymax={ymax}
boundary_type_xmin={bc[0]}
boundary_type_xmax={bc[1]}
boundary_type_ymin={bc[2]}
boundary_type_ymax={bc[3]}

[hydro]
gamma0={gamma0}
cfl={cfl}
niter_riemann=10
slope_type={slope_type}
problem={problem}
riemann={riemann}

{extra}
[other]
implementationVersion=0
"""


def write_ini(text: str, directory: str | None = None, name: str = "case.ini") -> str:
    d = directory or tempfile.mkdtemp(prefix="e2d_ini_")
    path = os.path.join(d, name)
    with open(path, "w") as f:
        f.write(text)
    return path


def smooth_state(nx, ny, gamma0, seed, *, amp=0.2):
    """A smooth positive state (rho, E, mx, my) of shape (4, ny+4, nx+4) built
    from a few seeded Fourier modes; exercises every branch of the limiter
    and of the Riemann solvers without shocks."""
    rng = np.random.default_rng(seed)
    isize, jsize = nx + 4, ny + 4
    x = (np.arange(isize) - 1.5) / nx
    y = (np.arange(jsize) - 1.5) / ny
    X, Y = np.meshgrid(x, y)
    def field(base):
        f = np.full_like(X, base)
        for _ in range(3):
            kx, ky = rng.integers(1, 4, size=2)
            ph = rng.uniform(0, 2 * np.pi)
            f += amp * base * rng.uniform(0.3, 1.0) * np.sin(2 * np.pi * (kx * X + ky * Y) + ph)
        return f
    rho = field(1.0)
    p = field(1.0)
    u = field(0.5) - 0.5
    v = field(0.5) - 0.5
    U = np.empty((4, jsize, isize))
    U[0] = rho
    U[2] = rho * u
    U[3] = rho * v
    U[1] = p / (gamma0 - 1.0) + 0.5 * rho * (u * u + v * v)
    return U


def implode_diag_state(nx, ny, gamma0, xmin=0.0, ymin=0.0, xmax=1.0, ymax=1.0):
    """The classic implosion split x + y > 0.5: rho=1, p=1 above, rho=0.125,
    p=0.14 below, at rest; cell centres as the reference computes them."""
    import struct

    f = lambda v: struct.unpack("f", struct.pack("f", float(v)))[0]
    xmin, xmax, ymin, ymax = f(xmin), f(xmax), f(ymin), f(ymax)
    dx = (xmax - xmin) / nx
    dy = (ymax - ymin) / ny
    isize, jsize = nx + 4, ny + 4
    U = np.zeros((4, jsize, isize))
    for j in range(jsize):
        for i in range(isize):
            x = xmin + dx / 2 + (i - 2) * dx
            y = ymin + dy / 2 + (j - 2) * dy
            inside = x + y > 0.5
            U[0, j, i] = 1.0 if inside else 0.125
            U[1, j, i] = (1.0 if inside else 0.14) / (gamma0 - 1.0)
    return U


def f32(v: float) -> float:
    import struct

    return struct.unpack("f", struct.pack("f", float(v)))[0]


# Multi-step run cases pinned against the reference.  Each entry:
#   name -> dict(ini=..., inject=callable or None, nsteps=int)
def run_cases():
    g14 = f32(1.4)
    cases = {
        # the reference's own implode ini (src/test_implode.ini physics), smaller grid
        "implode_ref_ini": dict(
            ini=ini_text(64, 32, problem="implode", gamma0=1.666, xmin=-1.0, xmax=1.0), inject=None,
            nsteps=40),
        "implode_diag": dict(ini=ini_text(48, 48, problem="implode"),
                             inject=lambda: implode_diag_state(48, 48, g14), nsteps=100),
        "blast_reflect": dict(
            ini=ini_text(48, 48, problem="blast",
                         extra="[blast]\nradius=0.125\ncenter_x=0.5\ncenter_y=0.5\ndensity_in=1.0\n"
                               "density_out=1.0\npressure_in=10.0\npressure_out=0.1\n"),
            inject=None, nsteps=60),
        "four_quadrant_absorb": dict(ini=ini_text(48, 48, bc=(2, 2, 2, 2), problem="four_quadrant"),
                                     inject=None, nsteps=60),
        "discontinuity_absorb": dict(ini=ini_text(40, 40, bc=(2, 2, 2, 2), problem="discontinuity",
                                                  gamma0=1.666), inject=None, nsteps=40),
        "periodic_smooth": dict(ini=ini_text(40, 36, bc=(3, 3, 3, 3)),
                                inject=lambda: smooth_state(40, 36, g14, seed=11), nsteps=50),
        "mixed_bc_smooth": dict(ini=ini_text(36, 44, bc=(1, 2, 3, 3)),
                                inject=lambda: smooth_state(36, 44, g14, seed=12), nsteps=40),
        "mixed_bc2_smooth": dict(ini=ini_text(34, 30, bc=(3, 3, 2, 1)),
                                 inject=lambda: smooth_state(34, 30, g14, seed=13), nsteps=40),
        "minmod_implode": dict(ini=ini_text(48, 40, problem="implode", slope_type=1),
                               inject=lambda: implode_diag_state(48, 40, g14), nsteps=40),
        "first_order_implode": dict(ini=ini_text(40, 48, problem="implode", slope_type=0),
                                    inject=lambda: implode_diag_state(40, 48, g14), nsteps=30),
        "shocked_bubble": dict(
            ini=ini_text(89, 18, bc=(2, 2, 1, 1), problem="shocked_bubble", gamma0=1.2, cfl=0.5,
                         xmax=0.445, ymax=0.089), inject=None, nsteps=30),
        "tend_clamp": dict(ini=ini_text(32, 32, problem="implode", tEnd=0.05, nStepmax=1000),
                           inject=lambda: implode_diag_state(32, 32, g14), nsteps=1000),
    }
    return cases


SEDOV_NBINS = (7, 40, 150)


def sedov_ini(nbins: int) -> str:
    """The physics of the reference's src/sedov_blast/test_sedov_blast_2d.ini
    (energy 0.311357 deposited in a disc, absorbing walls) on 64x64 cells,
    disc radius 0.05 so that it covers a few cells, 60 steps."""
    return ini_text(64, 64, bc=(2, 2, 2, 2), problem="blast", tEnd=0.5, nStepmax=60,
                    extra="[blast]\ndensity_in=1.0\ndensity_out=1.0\npressure_in=1\n"
                          "pressure_out=1e-7\nradius=0.05\ntotal_energy_inside=0.311357\n"
                          f"nbins={nbins}\n")


def parse_ini(text: str) -> dict:
    """'section.key' (lower case) -> value string, for the simple ini texts
    of these cases (comments, sections, key=value)."""
    out, section = {}, ""
    for raw in text.splitlines():
        line = raw.strip()
        if not line or line[0] in ";#":
            continue
        if line.startswith("["):
            section = line[1:line.index("]")]
            continue
        if "=" in line:
            k, v = line.split("=", 1)
            out[f"{section}.{k.strip()}".lower()] = v.split(" ;")[0].strip()
    return out


def oracle_kwargs(text: str) -> dict:
    """Arguments of oracle.pyoracle.make_params for an ini text, with the
    defaults of HydroParams::setup (src/HydroParams.cpp:42-156)."""
    m = parse_ini(text)
    g = lambda k, d: m.get(k, d)
    return dict(
        nx=int(g("mesh.nx", 2)), ny=int(g("mesh.ny", 2)),
        xmin=float(g("mesh.xmin", 0.0)), xmax=float(g("mesh.xmax", 1.0)),
        ymin=float(g("mesh.ymin", 0.0)), ymax=float(g("mesh.ymax", 1.0)),
        bc=tuple(int(g(f"mesh.boundary_type_{s}", 1)) for s in ("xmin", "xmax", "ymin", "ymax")),
        gamma0=float(g("hydro.gamma0", 1.4)), cfl=float(g("hydro.cfl", 0.5)),
        slope_type=float(g("hydro.slope_type", 1.0)),
        smallr=float(g("hydro.smallr", 1e-10)), smallc=float(g("hydro.smallc", 1e-10)),
        riemann=g("hydro.riemann", "approx"),
    )


def run_limits(text: str):
    m = parse_ini(text)
    return int(m.get("run.nstepmax", 1000)), f32(float(m.get("run.tend", 0.0)))


# A four-quadrant flow with drawn states (416 x 1824 cells, absorbing walls,
# split at 0.5, gamma 1.4, HLLC, CFL 0.8) on which FP32 arithmetic breaks
# down: the FP32C state turns non-finite near t = 0.048 on the column of the
# vertical split, and so does the reference's own single-precision build,
# near t = 0.05; FP64 runs it to the end (667 steps).
BREAKDOWN_NX, BREAKDOWN_NY = 416, 1824
BREAKDOWN_T_END = 0.07696256392150672
BREAKDOWN_STATES = [
    [1.4045364949998327, 1.2478185891339812, 1.0125626194788715, 1.4112208957238694],
    [0.5510051598548608, 1.3033349919491264, 1.4899767690701817, 0.8116696708168066],
    [1.9604589210178323, 0.12702456455098715, -1.1540322213586327, -0.050099086017271144],
    [1.3025418760856602, 1.7962252840716093, 0.2289799732296557, -1.1532139468078726],
]
