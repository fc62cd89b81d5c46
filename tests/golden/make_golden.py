"""Generates the golden fixtures of tests/golden/ by running the REFERENCE
solver itself: oracle/_ref/libe2d_ref.so, the reference's own HydroRun.h,
HydroRunFunctors.h, HydroBaseFunctor.h, HydroParams.cpp and ConfigMap/inih
sources compiled against a host-only Kokkos stand-in (oracle/Makefile).

Run where the reference tree is present:
    make -C oracle ref && python tests/golden/make_golden.py

Outputs (small, committed):
    params.json   HydroParams::setup results for a set of ini files
    kat.npz       per-function known answers (primitives, slopes, trace,
                  riemann_hllc, riemann_approx, make_boundaries, compute_dt)
    runs.npz      multi-step runs: dt of every step and the final state
    c1.json       the 256x256 implosion, 1000 steps: dt sequence and a
                  SHA-256 of the final state
    sedov.npz     the Sedov post-processing (src/main.cpp:175-179) of a 64x64
                  point blast after 60 steps: the .npy files the reference's
                  ComputeRadialProfileFunctor writes, for three ring counts
    impl.npz      the reference's implementations 1 and 2 on four run cases
    vtk.npz       HydroRun::saveVTK output: the .vti bytes of a 32x24 state
                  and the SHA-256 of the .vti of the C1 state

    python tests/golden/make_golden.py --only sedov   regenerates one file
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle.pyoracle import ReferenceLib  # noqa: E402
import _cases as C  # noqa: E402

PARAM_INIS = {
    "plain": C.ini_text(64, 48),
    "formatting": """; leading comment
# another comment
[RUN]
TEND = 2.5 ; inline comment after whitespace
nStepMax=0x20
nOutput=-1
[Mesh]
nx = 040
ny=24
xmin=-0.25
xmax=0.75
  ymin=7
boundary_type_xmin=3
boundary_type_xmax=3
boundary_type_ymin=2
boundary_type_ymax=1
[hydro]
gamma0=1.666
cfl=0.45
slope_type=1.0
smallc=1e-8
smallr=2e-9
riemann=not_a_solver
problem=blast
[blast]
radius=0.1;no space so part of the value
center_x=0.3
[OTHER]
implementationVersion=1.9
""",
    "defaults": "[mesh]\nnx=10\nny=12\n",
    "shocked_bubble": C.ini_text(89, 18, bc=(2, 2, 1, 1), problem="shocked_bubble", gamma0=1.2,
                                 cfl=0.5, xmax=0.445, ymax=0.089,
                                 extra="[shocked_bubble]\nbubble_pressure=1.0132\n"),
    "bad_impl": C.ini_text(16, 16, extra="[OTHER]\nimplementationVersion=7\n"),
    # every reading rule at once: a value continued on an indented line, a
    # line longer than 199 bytes (its tail read as a continuation), inline
    # ';' with and without whitespace before it, a line without '=', a
    # section header whose ']' follows a comment, tab separators
    "quirks": ("[run]\ntEnd=3.5\nnStepmax=77\n[mesh]\nnx=20\nny=10\n   30\n"
               "xmin=" + " " * 194 + "  -0.5\n"
               "xmax=2.0 ;comment\nymax=1.5;x\nymin=;0.25\n"
               "[hydro]\ngamma0=1.3\nthis line has no equals sign\ncfl = 0.3\n"
               "slope_type\t=\t1.0\t; tab comment\n[hydro ;broken]\nriemann=hll\nproblem=blast\n"
               "# comment\n; comment\nsmallr=1e-9\n\t\t2e-9\n[OTHER]\nimplementationVersion=1\n"),
}


def gen_params(R: ReferenceLib, tmp: str) -> dict:
    out = {}
    for name, text in PARAM_INIS.items():
        path = C.write_ini(text, tmp, f"p_{name}.ini")
        out[name] = {"ini": text, "params": R.params(path)}
    return out


def gen_kat(R: ReferenceLib, tmp: str) -> dict:
    rng = np.random.default_rng(2024)
    ini2 = C.write_ini(C.ini_text(16, 16, gamma0=1.4), tmp, "kat2.ini")
    ini1 = C.write_ini(C.ini_text(16, 16, gamma0=1.666, slope_type=1), tmp, "kat1.ini")
    kat = {"ini_slope2": np.array(open(ini2).read()), "ini_slope1": np.array(open(ini1).read())}
    n = 600
    # conservative states: ordinary, density below smallr, negative internal energy
    rho = np.exp(rng.uniform(np.log(1e-3), np.log(10.0), n))
    rho[:20] = rng.uniform(-1e-3, 1e-11, 20)
    u = rng.normal(0, 1.5, n)
    v = rng.normal(0, 1.5, n)
    p = np.exp(rng.uniform(np.log(1e-4), np.log(100.0), n))
    E = p / 0.4 + 0.5 * rho * (u * u + v * v)
    E[20:40] = 0.5 * rho[20:40] * (u[20:40] ** 2 + v[20:40] ** 2) * 0.9  # e < 0
    ucons = np.stack([rho, E, rho * u, rho * v], axis=1)
    ucons[40] = [1.0, 2.5, 0.0, -0.0]
    kat["prim_u"] = ucons
    kat["prim_q"], kat["prim_c"] = R.primitives(ini2, ucons)

    # slopes: random stencils, exact ties, sign changes, zero neighbours
    q5 = rng.normal(1.0, 0.5, (n, 5, 4))
    q5[:50, 1] = q5[:50, 0]          # drgt = 0
    q5[50:100, 2] = q5[50:100, 0]    # dlft = 0
    q5[100:150, 1] = 2 * q5[100:150, 0] - q5[100:150, 2]  # dcen == dlft exactly-ish
    q5[150:160] = 0.0
    kat["slope_q5"] = q5
    kat["slope2_dqx"], kat["slope2_dqy"] = R.slopes(ini2, q5)
    kat["slope1_dqx"], kat["slope1_dqy"] = R.slopes(ini1, q5)

    # traces on all four faces
    qt = np.stack([np.exp(rng.normal(0, 0.5, n)), np.exp(rng.normal(0, 0.5, n)),
                   rng.normal(0, 1, n), rng.normal(0, 1, n)], axis=1)
    dqx = rng.normal(0, 0.2, (n, 4))
    dqy = rng.normal(0, 0.2, (n, 4))
    dqx[:10, 0] = -50.0  # drives the face density below smallr
    kat["trace_q"], kat["trace_dqx"], kat["trace_dqy"] = qt, dqx, dqy
    kat["trace_dtdx"], kat["trace_dtdy"] = np.array(0.13), np.array(0.21)
    for face in range(4):
        kat[f"trace_face{face}"] = R.trace(ini2, qt, dqx, dqy, 0.13, 0.21, face)

    # Riemann problems: random, strong shocks, near vacuum, supersonic both
    # ways, at rest with u = +0/-0, identical states
    def states(m):
        return np.stack([np.exp(rng.normal(0, 1, m)), np.exp(rng.normal(0, 1.5, m)),
                         rng.normal(0, 2, m), rng.normal(0, 1, m)], axis=1)
    ql, qr = states(n), states(n)
    ql[:30, 2] = 8.0 + rng.uniform(0, 2, 30)     # SL > 0
    qr[30:60, 2] = -8.0 - rng.uniform(0, 2, 30)  # SR < 0
    ql[30:60, 2] = -9.0
    ql[60:90, 1] = 1e4
    qr[60:90, 1] = 1e-4                          # strong shock
    ql[90:120, 0] = 1e-9
    qr[90:120, 0] = 1e-9                         # near vacuum (smallr floor)
    ql[120:150, 2] = 0.0
    qr[120:150, 2] = -0.0                        # at rest, signed zeros
    ql[150:180] = qr[150:180]                    # identical states
    ql[180:200, 1] = -1.0                        # negative pressure (smallp floor)
    kat["riemann_ql"], kat["riemann_qr"] = ql, qr
    kat["riemann_hllc"] = R.riemann(ini2, "hllc", ql, qr)
    kat["riemann_approx"] = R.riemann(ini2, "approx", ql, qr)

    # make_boundaries and compute_dt for every boundary type on a random state
    for bcs in [(1, 1, 1, 1), (2, 2, 2, 2), (3, 3, 3, 3), (1, 2, 3, 1), (3, 1, 2, 3)]:
        tag = "".join(map(str, bcs))
        ini = C.write_ini(C.ini_text(7, 5, bc=bcs), tmp, f"bc{tag}.ini")
        u0 = C.smooth_state(7, 5, C.f32(1.4), seed=int(tag))
        u0 += rng.normal(0, 1e-3, u0.shape)  # distinct ghosts before the fill
        kat[f"bc{tag}_ini"] = np.array(open(ini).read())
        kat[f"bc{tag}_u0"] = u0
        kat[f"bc{tag}_u"] = R.make_boundaries(ini, u0)
        kat[f"bc{tag}_dt"] = np.array(R.compute_dt(ini, u0))
    return kat


def gen_runs(R: ReferenceLib, tmp: str) -> dict:
    out = {}
    for name, case in C.run_cases().items():
        path = C.write_ini(case["ini"], tmp, f"run_{name}.ini")
        u0 = case["inject"]() if case["inject"] else R.initial_state(path)
        u, dts, t, ns = R.run(path, u0 if case["inject"] else None, case["nsteps"])
        out[f"{name}__ini"] = np.array(case["ini"])
        out[f"{name}__u0"] = u0
        out[f"{name}__dt"] = dts
        out[f"{name}__u"] = u
        out[f"{name}__t"] = np.array(t)
        out[f"{name}__nsteps"] = np.array(ns)
        print(f"  run {name}: {ns} steps, t={t:.6g}")
    return out


def gen_c1(R: ReferenceLib, tmp: str) -> dict:
    """The implosion benchmark configuration: x+y>0.5, 256x256, gamma 1.4,
    CFL 0.8, reflecting walls, HLLC, 1000 steps."""
    text = C.ini_text(256, 256, problem="implode", nStepmax=1000)
    path = C.write_ini(text, tmp, "c1.ini")
    u0 = C.implode_diag_state(256, 256, C.f32(1.4))
    u, dts, t, ns = R.run(path, u0, 1000)
    interior = u[:, 2:-2, 2:-2]
    return {"ini": text, "nsteps": ns, "t": float(t).hex(),
            "dt_hex": [float(x).hex() for x in dts],
            "sha256_state": hashlib.sha256(np.ascontiguousarray(u).tobytes()).hexdigest(),
            "sum_interior": [float(interior[v].sum()).hex() for v in range(4)],
            "l1_interior": [float(np.abs(interior[v]).sum()).hex() for v in range(4)]}


IMPL_CASES = ("blast_reflect", "periodic_smooth", "mixed_bc_smooth", "implode_diag")


def gen_impl(R: ReferenceLib, tmp: str) -> dict:
    """The reference's implementations 1 and 2 ([OTHER] implementationVersion)
    on four of the run cases: dt of every step and the final state.  (The
    reference's implementation 2 adds fluxes with atomics; under OpenMP the
    order of those additions varies between runs at the rounding level.)"""
    out = {}
    cases = C.run_cases()
    for name in IMPL_CASES:
        case = cases[name]
        for impl in (1, 2):
            text = case["ini"] + f"\n[OTHER]\nimplementationVersion={impl}\n"
            path = C.write_ini(text, tmp, f"impl{impl}_{name}.ini")
            u0 = case["inject"]() if case["inject"] else None
            u, dts, t, ns = R.run(path, u0, case["nsteps"])
            key = f"{name}__impl{impl}"
            out[f"{key}__ini"] = np.array(text)
            out[f"{key}__t"] = np.array(t)
            out[f"{key}__nsteps"] = np.array(ns)
            if impl == 1:  # SHA-256 of the bits (they are implementation 0's: runs.npz)
                out[f"{key}__sha256"] = np.array(hashlib.sha256(np.ascontiguousarray(u).tobytes()
                                                                + np.ascontiguousarray(dts).tobytes()).hexdigest())
            else:
                out[f"{key}__dt"] = dts
                out[f"{key}__u"] = u
    return out


VTK_SMALL_INI = C.ini_text(32, 24, problem="implode", gamma0=1.666, xmin=-1.0, xmax=1.0)


def gen_vtk(R: ReferenceLib, tmp: str) -> dict:
    """HydroRun::saveVTK of the reference: the .vti bytes of a 32x24
    implosion on [-1,1]x[0,1] after 20 steps from its own initial condition
    (state included), and the SHA-256 of the .vti of the 256^2 implosion
    after 1000 steps (the C1 state)."""
    out = {"small_ini": np.array(VTK_SMALL_INI)}
    outdir = os.path.join(tmp, "vtk")
    os.makedirs(outdir, exist_ok=True)
    section = f"\n[output]\noutputDir={outdir}\noutputPrefix=ref\n"
    path = C.write_ini(VTK_SMALL_INI + section, tmp, "vtk_small.ini")
    u, _, _, ns = R.run(path, None, 20)
    R.save_vtk(path, u, ns)
    out["small_u"] = u
    out["small_nsteps"] = np.array(ns)
    out["small_vti"] = np.frombuffer(open(os.path.join(outdir, f"ref_{ns:07d}.vti"), "rb").read(), dtype=np.uint8)
    text = C.ini_text(256, 256, problem="implode", nStepmax=1000)
    path = C.write_ini(text + section, tmp, "vtk_c1.ini")
    u, _, _, ns = R.run(path, C.implode_diag_state(256, 256, C.f32(1.4)), 1000)
    R.save_vtk(path, u, ns)
    vti = open(os.path.join(outdir, f"ref_{ns:07d}.vti"), "rb").read()
    out["c1_vti_sha256"] = np.array(hashlib.sha256(vti).hexdigest())
    out["c1_vti_bytes"] = np.array(len(vti))
    return out


def gen_sedov(R: ReferenceLib, tmp: str) -> dict:
    """The reference's own initial condition and 60 steps, then its radial
    profile with 7, 40 and 150 rings: the raw bytes of both .npy files."""
    path = C.write_ini(C.sedov_ini(C.SEDOV_NBINS[0]), tmp, "sedov.ini")
    u, dts, t, ns = R.run(path, None, 60)
    out = {"nsteps": np.int64(ns), "rho": u[0], "dt": dts,
           "sha256_state": np.frombuffer(hashlib.sha256(np.ascontiguousarray(u).tobytes()).digest(),
                                         dtype=np.uint8)}
    for nb in C.SEDOV_NBINS:
        pb = C.write_ini(C.sedov_ini(nb), tmp, f"sedov_{nb}.ini")
        dist, prof = R.radial_profile(pb, u)
        out[f"dist_npy_{nb}"] = np.frombuffer(dist, dtype=np.uint8)
        out[f"prof_npy_{nb}"] = np.frombuffer(prof, dtype=np.uint8)
    return out


def main():
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["params", "kat", "runs", "c1", "sedov", "vtk", "impl"])
    only = ap.parse_args().only
    R = ReferenceLib()
    tmp = tempfile.mkdtemp(prefix="e2d_golden_")
    if only in (None, "params"):
        with open(os.path.join(HERE, "params.json"), "w") as f:
            json.dump(gen_params(R, tmp), f, indent=1)
    if only in (None, "kat"):
        np.savez_compressed(os.path.join(HERE, "kat.npz"), **gen_kat(R, tmp))
    if only in (None, "runs"):
        np.savez_compressed(os.path.join(HERE, "runs.npz"), **gen_runs(R, tmp))
    if only in (None, "c1"):
        with open(os.path.join(HERE, "c1.json"), "w") as f:
            json.dump(gen_c1(R, tmp), f, indent=1)
    if only in (None, "impl"):
        np.savez_compressed(os.path.join(HERE, "impl.npz"), **gen_impl(R, tmp))
    if only in (None, "vtk"):
        np.savez_compressed(os.path.join(HERE, "vtk.npz"), **gen_vtk(R, tmp))
    if only in (None, "sedov"):
        np.savez_compressed(os.path.join(HERE, "sedov.npz"), **gen_sedov(R, tmp))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
