"""ctypes front end of the CPU oracle (oracle/e2d_oracle.c).

Test infrastructure only: tests/, the smoke check and the benchmark's CPU
baseline use it as the parity checker for the GPU path; the product never
imports it.  `ReferenceLib` wraps oracle/_ref/libe2d_ref.so, the reference's
own solver sources compiled against a host-only Kokkos stand-in; it exists
only where the reference tree is present and is used to pin the oracle.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libe2d_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libe2d_ref.so")

RIEMANN = {"approx": 0, "hll": 1, "hllc": 2}


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("ghost", ctypes.c_int),
        ("isize", ctypes.c_int), ("jsize", ctypes.c_int),
        ("xmin", ctypes.c_double), ("xmax", ctypes.c_double),
        ("ymin", ctypes.c_double), ("ymax", ctypes.c_double),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double),
        ("bc_xmin", ctypes.c_int), ("bc_xmax", ctypes.c_int),
        ("bc_ymin", ctypes.c_int), ("bc_ymax", ctypes.c_int),
        ("gamma0", ctypes.c_double), ("gamma6", ctypes.c_double), ("cfl", ctypes.c_double),
        ("slope_type", ctypes.c_double), ("smallr", ctypes.c_double),
        ("smallc", ctypes.c_double), ("smallp", ctypes.c_double), ("smallpp", ctypes.c_double),
        ("riemann", ctypes.c_int),
    ]


def f32(x: float) -> float:
    """Value of a real ini parameter as ConfigMap::getFloat returns it
    (config/ConfigMap.cpp:31-40 parses with strtof into a float)."""
    return struct.unpack("f", struct.pack("f", float(x)))[0]


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        P = ctypes.POINTER(OrcParams)
        dp = ctypes.c_void_p
        L.orc_params_init.argtypes = [P]
        L.orc_primitives.argtypes = [P, dp, dp, dp]
        L.orc_slopes.argtypes = [P, dp, dp, dp, dp, dp, dp, dp]
        L.orc_trace.argtypes = [P, dp, dp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_int, dp]
        L.orc_riemann.argtypes = [P, ctypes.c_int, dp, dp, dp]
        L.orc_make_boundaries.argtypes = [P, dp]
        L.orc_compute_dt.argtypes = [P, dp]
        L.orc_compute_dt.restype = ctypes.c_double
        L.orc_godunov_step.argtypes = [P, dp, dp, ctypes.c_double, dp]
        L.orc_run.argtypes = [P, dp, dp, ctypes.c_int, ctypes.c_double, dp, dp]
        L.orc_run.restype = ctypes.c_int
        L.orc_init_implode.argtypes = [P, dp, ctypes.c_int]
        L.orc_init_blast.argtypes = [P, dp] + [ctypes.c_double] * 7
        L.orc_init_four_quadrant.argtypes = [P, dp, ctypes.c_double, ctypes.c_double, dp]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_radial_profile.argtypes = [P, dp, ctypes.c_int, dp, dp, dp]
        _lib = L
    return _lib


def make_params(nx, ny, *, gamma0=1.4, cfl=0.8, slope_type=2.0, smallr=1e-10, smallc=1e-10,
                bc=(1, 1, 1, 1), riemann="hllc", xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0,
                float_params=True) -> OrcParams:
    """HydroParams as HydroParams::setup builds it (src/HydroParams.cpp:42-156).
    With float_params the real values go through float like ConfigMap does."""
    cv = f32 if float_params else float
    p = OrcParams()
    p.nx, p.ny = int(nx), int(ny)
    p.xmin, p.xmax, p.ymin, p.ymax = cv(xmin), cv(xmax), cv(ymin), cv(ymax)
    p.bc_xmin, p.bc_xmax, p.bc_ymin, p.bc_ymax = (int(b) for b in bc)
    p.gamma0, p.cfl, p.slope_type = cv(gamma0), cv(cfl), cv(slope_type)
    p.smallr, p.smallc = cv(smallr), cv(smallc)
    p.riemann = RIEMANN[riemann] if isinstance(riemann, str) else int(riemann)
    lib().orc_params_init(ctypes.byref(p))
    return p


def new_state(p: OrcParams) -> np.ndarray:
    """A zeroed (4, jsize, isize) C-contiguous array: LayoutLeft memory order."""
    return np.zeros((4, p.jsize, p.isize), dtype=np.float64)


def _ptr(a: np.ndarray):
    assert a.flags.c_contiguous and a.dtype == np.float64
    return a.ctypes.data_as(ctypes.c_void_p)


def init_implode(p, reference_shape=False):
    u = new_state(p)
    lib().orc_init_implode(ctypes.byref(p), _ptr(u), int(reference_shape))
    return u


def init_blast(p, radius=0.125, cx=0.5, cy=0.5, d_in=1.0, d_out=1.0, p_in=10.0, p_out=0.1):
    u = new_state(p)
    lib().orc_init_blast(ctypes.byref(p), _ptr(u), radius, cx, cy, d_in, d_out, p_in, p_out)
    return u


LAX_LIU_3 = np.array([1.5, 1.5, 0.0, 0.0,
                      0.5323, 0.3, 1.206, 0.0,
                      0.138, 0.029, 1.206, 1.206,
                      0.5323, 0.3, 0.0, 1.206], dtype=np.float64)


def init_four_quadrant(p, xt=0.5, yt=0.5, prim=LAX_LIU_3):
    u = new_state(p)
    prim = np.ascontiguousarray(prim, dtype=np.float64)
    lib().orc_init_four_quadrant(ctypes.byref(p), _ptr(u), xt, yt, _ptr(prim))
    return u


def run(p, u0, nstep_max, t_end):
    """The reference main loop from u0; returns (state, dt_trace, t, nsteps)."""
    u = np.array(u0, dtype=np.float64, order="C", copy=True)
    u2 = u.copy()
    dts = np.zeros(max(int(nstep_max), 1))
    t = ctypes.c_double()
    ns = lib().orc_run(ctypes.byref(p), _ptr(u), _ptr(u2), int(nstep_max), float(t_end),
                       _ptr(dts), ctypes.cast(ctypes.byref(t), ctypes.c_void_p))
    cur = u if ns % 2 == 0 else u2
    return cur, dts[:ns], t.value, ns


def compute_dt(p, u):
    return lib().orc_compute_dt(ctypes.byref(p), _ptr(np.ascontiguousarray(u)))


def make_boundaries(p, u):
    u = np.array(u, dtype=np.float64, order="C", copy=True)
    lib().orc_make_boundaries(ctypes.byref(p), _ptr(u))
    return u


def godunov_step(p, u_in, dt):
    """One godunov_unsplit_impl call; returns (u_in after the ghost fill, u_out)."""
    u_in = np.array(u_in, dtype=np.float64, order="C", copy=True)
    u_out = np.zeros_like(u_in)
    work = np.zeros((12,) + u_in.shape[1:])
    lib().orc_godunov_step(ctypes.byref(p), _ptr(u_in), _ptr(u_out), float(dt), _ptr(work))
    return u_in, u_out


def primitives(p, u):
    u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1, 4)
    q = np.zeros_like(u)
    c = np.zeros(len(u))
    for k in range(len(u)):
        lib().orc_primitives(ctypes.byref(p), _ptr(u[k]), _ptr(q[k]),
                             c[k:k + 1].ctypes.data_as(ctypes.c_void_p))
    return q, c


def slopes(p, q5):
    q5 = np.ascontiguousarray(q5, dtype=np.float64).reshape(-1, 5, 4)
    dqx = np.zeros((len(q5), 4))
    dqy = np.zeros((len(q5), 4))
    for k in range(len(q5)):
        s = [np.ascontiguousarray(q5[k, m]) for m in range(5)]
        lib().orc_slopes(ctypes.byref(p), *[_ptr(x) for x in s], _ptr(dqx[k]), _ptr(dqy[k]))
    return dqx, dqy


def trace(p, q, dqx, dqy, dtdx, dtdy, face):
    q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 4)
    dqx = np.ascontiguousarray(dqx, dtype=np.float64).reshape(-1, 4)
    dqy = np.ascontiguousarray(dqy, dtype=np.float64).reshape(-1, 4)
    out = np.zeros_like(q)
    for k in range(len(q)):
        lib().orc_trace(ctypes.byref(p), _ptr(q[k]), _ptr(dqx[k]), _ptr(dqy[k]),
                        dtdx, dtdy, int(face), _ptr(out[k]))
    return out


def riemann(p, solver, ql, qr):
    ql = np.ascontiguousarray(ql, dtype=np.float64).reshape(-1, 4)
    qr = np.ascontiguousarray(qr, dtype=np.float64).reshape(-1, 4)
    out = np.zeros_like(ql)
    s = RIEMANN[solver] if isinstance(solver, str) else int(solver)
    for k in range(len(ql)):
        lib().orc_riemann(ctypes.byref(p), s, _ptr(ql[k]), _ptr(qr[k]), _ptr(out[k]))
    return out


def radial_profile(p, u, nbins):
    """(distances, mean density, cell count) per ring -- orc_radial_profile."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    d, prof = np.zeros(nbins), np.zeros(nbins)
    cnt = np.zeros(nbins, dtype=np.int64)
    lib().orc_radial_profile(ctypes.byref(p), _ptr(u), int(nbins), _ptr(d), _ptr(prof),
                             cnt.ctypes.data_as(ctypes.c_void_p))
    return d, prof, cnt


class ReferenceLib:
    """The reference's own solver (oracle/_ref/libe2d_ref.so), driven by ini files."""

    def __init__(self, path: str = REF_SO):
        L = ctypes.CDLL(path)
        dp = ctypes.c_void_p
        L.ref_params.argtypes = [ctypes.c_char_p, dp]
        L.ref_run.argtypes = [ctypes.c_char_p, dp, ctypes.c_int, dp, dp,
                              ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
        L.ref_initial_state.argtypes = [ctypes.c_char_p, dp]
        L.ref_make_boundaries.argtypes = [ctypes.c_char_p, dp]
        L.ref_save_vtk.argtypes = [ctypes.c_char_p, dp, ctypes.c_int]
        L.ref_compute_dt.argtypes = [ctypes.c_char_p, dp]
        L.ref_compute_dt.restype = ctypes.c_double
        L.ref_primitives.argtypes = [ctypes.c_char_p, ctypes.c_int, dp, dp, dp]
        L.ref_slopes.argtypes = [ctypes.c_char_p, ctypes.c_int, dp, dp, dp]
        L.ref_trace.argtypes = [ctypes.c_char_p, ctypes.c_int, dp, dp, dp,
                                ctypes.c_double, ctypes.c_double, ctypes.c_int, dp]
        L.ref_riemann.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, dp, dp, dp]
        L.ref_radial_profile.argtypes = [ctypes.c_char_p, dp, ctypes.c_char_p]
        L.ref_radial_profile.restype = ctypes.c_int
        self.L = L

    def radial_profile(self, ini: str, u):
        """The reference's Sedov post-processing on state u: returns the bytes
        of the two .npy files it writes (distances, density profile)."""
        import tempfile

        u = np.ascontiguousarray(u, dtype=np.float64)
        with tempfile.TemporaryDirectory() as d:
            if self.L.ref_radial_profile(ini.encode(), _ptr(u), d.encode()) != 0:
                raise RuntimeError("ref_radial_profile failed")
            out = []
            for name in ("sedov_blast_radial_distances.npy", "sedov_blast_density_profile.npy"):
                with open(os.path.join(d, name), "rb") as f:
                    out.append(f.read())
        return tuple(out)

    PARAM_NAMES = ["nx", "ny", "isize", "jsize", "dx", "dy", "gamma0", "gamma6", "cfl",
                   "slope_type", "smallr", "smallc", "smallp", "smallpp", "tEnd", "nStepmax",
                   "bc_xmin", "bc_xmax", "bc_ymin", "bc_ymax", "riemann", "problem", "impl",
                   "xmin", "xmax", "ymin", "ymax"]

    def params(self, ini: str) -> dict:
        out = np.zeros(64)
        n = self.L.ref_params(ini.encode(), _ptr(out))
        return dict(zip(self.PARAM_NAMES, out[:n].tolist()))

    def run(self, ini: str, u0=None, nstep_limit=-1):
        pr = self.params(ini)
        isize, jsize = int(pr["isize"]), int(pr["jsize"])
        nmax = int(pr["nStepmax"]) if nstep_limit < 0 else nstep_limit
        u = np.zeros((4, jsize, isize))
        dts = np.zeros(max(nmax, 1))
        ns = ctypes.c_int()
        t = ctypes.c_double()
        u0p = None if u0 is None else _ptr(np.ascontiguousarray(u0, dtype=np.float64))
        self.L.ref_run(ini.encode(), u0p, int(nstep_limit), _ptr(u), _ptr(dts),
                       ctypes.byref(ns), ctypes.byref(t))
        return u, dts[:ns.value], t.value, ns.value

    def initial_state(self, ini: str):
        pr = self.params(ini)
        u = np.zeros((4, int(pr["jsize"]), int(pr["isize"])))
        self.L.ref_initial_state(ini.encode(), _ptr(u))
        return u

    def make_boundaries(self, ini: str, u):
        u = np.array(u, dtype=np.float64, order="C", copy=True)
        self.L.ref_make_boundaries(ini.encode(), _ptr(u))
        return u

    def save_vtk(self, ini: str, u, istep: int):
        """HydroRun::saveData(U, istep) of the reference on state u: the .vti
        file named by the ini's [output] outputDir and outputPrefix."""
        self.L.ref_save_vtk(ini.encode(), _ptr(np.ascontiguousarray(u, dtype=np.float64)), int(istep))

    def compute_dt(self, ini: str, u):
        return self.L.ref_compute_dt(ini.encode(), _ptr(np.ascontiguousarray(u)))

    def primitives(self, ini, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1, 4)
        q = np.zeros_like(u)
        c = np.zeros(len(u))
        self.L.ref_primitives(ini.encode(), len(u), _ptr(u), _ptr(q), _ptr(c))
        return q, c

    def slopes(self, ini, q5):
        q5 = np.ascontiguousarray(q5, dtype=np.float64).reshape(-1, 5, 4)
        dqx = np.zeros((len(q5), 4))
        dqy = np.zeros((len(q5), 4))
        self.L.ref_slopes(ini.encode(), len(q5), _ptr(q5), _ptr(dqx), _ptr(dqy))
        return dqx, dqy

    def trace(self, ini, q, dqx, dqy, dtdx, dtdy, face):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 4)
        out = np.zeros_like(q)
        self.L.ref_trace(ini.encode(), len(q), _ptr(q),
                         _ptr(np.ascontiguousarray(dqx, dtype=np.float64).reshape(-1, 4)),
                         _ptr(np.ascontiguousarray(dqy, dtype=np.float64).reshape(-1, 4)),
                         dtdx, dtdy, int(face), _ptr(out))
        return out

    def riemann(self, ini, solver, ql, qr):
        ql = np.ascontiguousarray(ql, dtype=np.float64).reshape(-1, 4)
        qr = np.ascontiguousarray(qr, dtype=np.float64).reshape(-1, 4)
        out = np.zeros_like(ql)
        s = RIEMANN[solver] if isinstance(solver, str) else int(solver)
        self.L.ref_riemann(ini.encode(), s, len(ql), _ptr(ql), _ptr(qr), _ptr(out))
        return out
