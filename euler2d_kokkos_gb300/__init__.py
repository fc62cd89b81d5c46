"""GB300-native unsplit MUSCL-Hancock Godunov step of euler2d_kokkos.

Python front end of the C ABI in include/e2d.h (libe2d_gb300.so, built
in-tree by euler2d_kokkos_gb300/build.py).  It mirrors the reference's
driver interface:

    params = HydroParams.from_ini("test_implode.ini")    # ConfigMap + HydroParams::setup
    hydro  = HydroRun(params)                              # HydroRun<device>(params, configMap)
    dt     = hydro.compute_dt(nStep % 2)
    hydro.godunov_unsplit(nStep, dt)

and adds the device-resident time loop (`step_n`).  All computation runs in
hand-written sm_103a kernels; there is no CPU fallback: importing this module
fails if the library cannot be loaded.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

__all__ = ["HydroParams", "HydroRun", "E2DError", "load_library", "ID", "IP", "IE", "IU", "IV",
           "RIEMANN", "BC_REFLECT", "BC_ABSORB", "BC_PERIODIC", "PROBLEMS", "PRECISION_FP64",
           "PRECISION_FP32C", "PRECISION_FP64_FAST"]

ID, IP, IE, IU, IV = 0, 1, 1, 2, 3
RIEMANN = {"approx": 0, "hll": 1, "hllc": 2}
BC_REFLECT, BC_ABSORB, BC_PERIODIC = 1, 2, 3
PROBLEMS = {"implode": 0, "blast": 1, "four_quadrant": 2, "discontinuity": 3, "shocked_bubble": 4}
PRECISION_FP64, PRECISION_FP32C, PRECISION_FP64_FAST = 0, 1, 2
LAYOUT_LEFT, LAYOUT_RIGHT = 0, 1

STATUS = {0: "E2D_OK", 1: "E2D_EINVAL", 2: "E2D_ENOMEM", 3: "E2D_ENUMERIC", 4: "E2D_ETIMEOUT",
          5: "E2D_ECUDA", 6: "E2D_EIO"}


class E2DError(RuntimeError):
    """A non-zero e2d_status from the library."""

    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = f"{where}: {STATUS.get(status, status)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


class _Params(ctypes.Structure):
    # field order of struct e2d_params (include/e2d.h)
    _fields_ = [
        ("nStepmax", ctypes.c_int), ("tEnd", ctypes.c_double), ("nOutput", ctypes.c_int),
        ("enableOutput", ctypes.c_int), ("ioVTK", ctypes.c_int), ("ioHDF5", ctypes.c_int),
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("ghostWidth", ctypes.c_int),
        ("xmin", ctypes.c_double), ("xmax", ctypes.c_double),
        ("ymin", ctypes.c_double), ("ymax", ctypes.c_double),
        ("boundary_type_xmin", ctypes.c_int), ("boundary_type_xmax", ctypes.c_int),
        ("boundary_type_ymin", ctypes.c_int), ("boundary_type_ymax", ctypes.c_int),
        ("gamma0", ctypes.c_double), ("cfl", ctypes.c_double), ("slope_type", ctypes.c_double),
        ("smallr", ctypes.c_double), ("smallc", ctypes.c_double),
        ("niter_riemann", ctypes.c_int), ("riemannSolverType", ctypes.c_int),
        ("problemType", ctypes.c_int),
        ("blast_radius", ctypes.c_double), ("blast_center_x", ctypes.c_double),
        ("blast_center_y", ctypes.c_double), ("blast_density_in", ctypes.c_double),
        ("blast_density_out", ctypes.c_double), ("blast_pressure_in", ctypes.c_double),
        ("blast_pressure_out", ctypes.c_double), ("blast_total_energy_inside", ctypes.c_double),
        ("blast_nbins", ctypes.c_int),
        ("bubble_radius", ctypes.c_double), ("bubble_center_x", ctypes.c_double),
        ("bubble_center_y", ctypes.c_double), ("bubble_density", ctypes.c_double),
        ("bubble_pressure", ctypes.c_double), ("preshock_density", ctypes.c_double),
        ("preshock_pressure", ctypes.c_double), ("postshock_density", ctypes.c_double),
        ("postshock_pressure", ctypes.c_double), ("postshock_velocity", ctypes.c_double),
        ("shock_loc", ctypes.c_double),
        ("fq_split_x", ctypes.c_double), ("fq_split_y", ctypes.c_double),
        ("fq_state", (ctypes.c_double * 4) * 4),
        ("implode_shape", ctypes.c_int),
        ("implementationVersion", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("imin", ctypes.c_int), ("imax", ctypes.c_int), ("jmin", ctypes.c_int),
        ("jmax", ctypes.c_int), ("isize", ctypes.c_int), ("jsize", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("smallp", ctypes.c_double),
        ("smallpp", ctypes.c_double), ("gamma6", ctypes.c_double),
    ]


# Every symbol declared in include/e2d.h, with its ctypes signature.
_P = ctypes.POINTER(_Params)
_V = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
SIGNATURES = {
    "e2d_abi_version": ([], _I),
    "e2d_status_string": ([_I], ctypes.c_char_p),
    "e2d_params_defaults": ([_P], _I),
    "e2d_params_from_ini": ([ctypes.c_char_p, _P], _I),
    "e2d_params_init": ([_P], _I),
    "e2d_ini_get_string": ([ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                            ctypes.c_char_p, ctypes.c_size_t], _I),
    "e2d_save_vtk": ([_V, _I, ctypes.c_char_p], _I),
    "e2d_write_vtk": ([_P, _V, _I, ctypes.c_char_p], _I),
    "e2d_fp64_rates": ([_V], _I),
    "e2d_create": ([_P, ctypes.POINTER(_V)], _I),
    "e2d_destroy": ([_V], _I),
    "e2d_last_error": ([_V], ctypes.c_char_p),
    "e2d_get_params": ([_V, _P], _I),
    "e2d_init_problem": ([_V], _I),
    "e2d_set_state": ([_V, _I, _V, _I], _I),
    "e2d_get_state": ([_V, _I, _V, _I], _I),
    "e2d_device_state": ([_V, _I, ctypes.POINTER(_V)], _I),
    "e2d_get_stream": ([_V, ctypes.POINTER(_V)], _I),
    "e2d_make_boundaries": ([_V, _I], _I),
    "e2d_compute_dt": ([_V, _I, ctypes.POINTER(_D)], _I),
    "e2d_godunov_unsplit": ([_V, _I, _D], _I),
    "e2d_godunov_unsplit_noalloc": ([_P, _V, _V, _D, _V], _I),
    "e2d_step_n": ([_V, _I, _D, ctypes.POINTER(_D), ctypes.POINTER(_I), _V], _I),
    "e2d_eval_device": ([_P, _I, _I, _V, _V, _D, _D], _I),
    "e2d_conservation": ([_V, _I, _V], _I),
    "e2d_l1_diff": ([_V, _I, _V, _I, _I, ctypes.POINTER(_D), ctypes.POINTER(_D)], _I),
    "e2d_radial_profile": ([_V, _I, _I, _V, _V, _V], _I),
    "e2d_save_npy": ([ctypes.c_char_p, _V, ctypes.c_longlong], _I),
    "e2d_batch_create": ([_I, ctypes.c_size_t, _I, ctypes.POINTER(_V)], _I),
    "e2d_batch_destroy": ([_V], _I),
    "e2d_batch_last_error": ([_V], ctypes.c_char_p),
    "e2d_batch_instance_bytes": ([_P], ctypes.c_size_t),
    "e2d_batch_free_bytes": ([_V, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)], _I),
    "e2d_batch_admit": ([_V, _P, _D, _V, ctypes.POINTER(_I)], _I),
    "e2d_batch_run": ([_V, _I, ctypes.POINTER(_I)], _I),
    "e2d_batch_query": ([_V, _I, ctypes.POINTER(_D), ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
    "e2d_batch_get_state": ([_V, _I, _V, _I], _I),
    "e2d_batch_release": ([_V, _I], _I),
    "e2d_batch_stats": ([_V, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(_I)], _I),
    "e2d_batch_stream": ([_V, ctypes.POINTER(_V)], _I),
    "e2d_batch_set_tuning": ([_V, _I, _V], _I),
    "e2d_batch_get_tuning": ([_V, ctypes.POINTER(_I), _V], _I),
    "e2d_batch_autotune": ([_V, _I], _I),
    "e2d_set_profiling": ([_V, _I], _I),
    "e2d_kernel_times": ([_V, _I, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(_D),
                          ctypes.POINTER(ctypes.c_long), ctypes.POINTER(_I)], _I),
    "e2d_reset_kernel_times": ([_V], _I),
}

_lib = None
ABI_VERSION = 2  # E2D_ABI_VERSION of include/e2d.h: the layout of _Params


def load_library(path: str | None = None, build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libe2d_gb300.so (building it first if it is absent) and bind
    every entry point of include/e2d.h.  Raises if anything is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    so = path or _build.LIB
    if not os.path.exists(so):
        if not build_if_missing:
            raise OSError(f"{so} not found; run euler2d_kokkos_gb300/build.py")
        _build.build()
    L = ctypes.CDLL(so)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(L, name)  # AttributeError if the library lacks a symbol
        fn.argtypes = args
        fn.restype = res
    if L.e2d_abi_version() != ABI_VERSION:
        raise OSError(f"{so}: ABI version {L.e2d_abi_version()}, this binding expects {ABI_VERSION}; rebuild it")
    if path is None:
        _lib = L
    return L


def _check(status: int, where: str, sim=None):
    if status != 0:
        detail = ""
        if sim is not None:
            detail = (load_library().e2d_last_error(sim) or b"").decode()
        raise E2DError(status, where, detail)


class HydroParams:
    """HydroParams + HydroSettings (src/HydroParams.h:107-265) as the flat
    e2d_params struct.  Attribute access reads/writes the struct fields."""

    def __init__(self, raw: _Params | None = None):
        object.__setattr__(self, "_raw", raw if raw is not None else _Params())
        if raw is None:
            load_library().e2d_params_defaults(ctypes.byref(self._raw))

    @classmethod
    def from_ini(cls, path: str) -> "HydroParams":
        """ConfigMap(path) followed by HydroParams::setup (reals go through float)."""
        p = cls()
        _check(load_library().e2d_params_from_ini(os.fsencode(path), ctypes.byref(p._raw)),
               f"params_from_ini({path})")
        return p

    def init(self) -> "HydroParams":
        """HydroParams::init: derived sizes and cut-offs, with validation."""
        _check(load_library().e2d_params_init(ctypes.byref(self._raw)), "params_init")
        return self

    def copy(self) -> "HydroParams":
        raw = _Params()
        ctypes.memmove(ctypes.byref(raw), ctypes.byref(self._raw), ctypes.sizeof(_Params))
        return HydroParams(raw)

    def __getattr__(self, name):
        return getattr(object.__getattribute__(self, "_raw"), name)

    def __setattr__(self, name, value):
        setattr(self._raw, name, value)

    def as_dict(self) -> dict:
        return {f: getattr(self._raw, f) for f, _ in _Params._fields_}


def make_params(nx, ny, *, problem="implode", riemann="hllc", gamma0=1.4, cfl=0.8,
                slope_type=2.0, bc=(1, 1, 1, 1), xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0,
                smallr=1e-10, smallc=1e-10, precision=PRECISION_FP64, float_params=True,
                **extra) -> HydroParams:
    """Parameters as HydroParams::setup would build them from an ini file
    holding these values (with float_params, reals are rounded through float
    like ConfigMap::getFloat)."""
    import struct as _st

    cv = (lambda x: _st.unpack("f", _st.pack("f", float(x)))[0]) if float_params else float
    p = HydroParams()
    p.nx, p.ny = int(nx), int(ny)
    p.xmin, p.xmax, p.ymin, p.ymax = cv(xmin), cv(xmax), cv(ymin), cv(ymax)
    (p.boundary_type_xmin, p.boundary_type_xmax,
     p.boundary_type_ymin, p.boundary_type_ymax) = (int(b) for b in bc)
    p.gamma0, p.cfl, p.slope_type = cv(gamma0), cv(cfl), cv(slope_type)
    p.smallr, p.smallc = cv(smallr), cv(smallc)
    p.riemannSolverType = RIEMANN[riemann] if isinstance(riemann, str) else int(riemann)
    p.problemType = PROBLEMS[problem] if isinstance(problem, str) else int(problem)
    p.precision = int(precision)
    for k, v in extra.items():
        setattr(p, k, cv(v) if isinstance(v, float) else v)
    return p.init()


class HydroRun:
    """HydroRun<device> (src/HydroRun.h:44-134) on one GB300.

    Owns U and U2 on the device.  `compute_dt`, `godunov_unsplit` and
    `make_boundaries` follow the reference's methods; `U`/`U2` return host
    copies shaped (4, jsize, isize) -- the reference's LayoutLeft memory
    order with v = (rho, E, mx, my)."""

    def __init__(self, params: HydroParams, init_problem: bool = True):
        self._lib = load_library()
        self.params = params.copy()
        h = ctypes.c_void_p()
        _check(self._lib.e2d_create(ctypes.byref(self.params._raw), ctypes.byref(h)), "e2d_create")
        self._h = h
        raw = _Params()
        self._lib.e2d_get_params(self._h, ctypes.byref(raw))
        self.params = HydroParams(raw)
        self.shape = (4, self.params.jsize, self.params.isize)
        if init_problem:
            _check(self._lib.e2d_init_problem(self._h), "e2d_init_problem", self._h)

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            self._lib.e2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- state transfer
    def set_state(self, which: int, u: np.ndarray, layout: int = LAYOUT_LEFT):
        u = np.ascontiguousarray(u, dtype=np.float64)
        if u.size != int(np.prod(self.shape)):
            raise ValueError(f"state has {u.size} values, expected {int(np.prod(self.shape))}")
        _check(self._lib.e2d_set_state(self._h, int(which), u.ctypes.data, layout), "e2d_set_state", self._h)

    def get_state(self, which: int, out: np.ndarray | None = None, layout: int = LAYOUT_LEFT):
        if out is None:
            out = np.empty(self.shape if layout == LAYOUT_LEFT
                           else (self.params.isize, self.params.jsize, 4), dtype=np.float64)
        _check(self._lib.e2d_get_state(self._h, int(which), out.ctypes.data, layout), "e2d_get_state", self._h)
        return out

    def save_vtk(self, which: int, filename: str) -> None:
        """HydroRun::saveVTK (src/HydroRun.h:506-609): state `which` as an
        ASCII .vti file of the interior cells, the reference's text format."""
        _check(self._lib.e2d_save_vtk(self._h, int(which), os.fsencode(filename)), "e2d_save_vtk", self._h)

    @property
    def U(self) -> np.ndarray:
        return self.get_state(0)

    @property
    def U2(self) -> np.ndarray:
        return self.get_state(1)

    def device_state(self, which: int) -> int:
        ptr = ctypes.c_void_p()
        _check(self._lib.e2d_device_state(self._h, int(which), ctypes.byref(ptr)), "e2d_device_state")
        return ptr.value

    def stream(self) -> int:
        ptr = ctypes.c_void_p()
        _check(self._lib.e2d_get_stream(self._h, ctypes.byref(ptr)), "e2d_get_stream")
        return ptr.value or 0

    # -- the reference's methods
    def make_boundaries(self, which: int):
        _check(self._lib.e2d_make_boundaries(self._h, int(which)), "make_boundaries", self._h)

    def compute_dt(self, useU: int) -> float:
        dt = ctypes.c_double()
        _check(self._lib.e2d_compute_dt(self._h, int(useU), ctypes.byref(dt)), "compute_dt", self._h)
        return dt.value

    def godunov_unsplit(self, nStep: int, dt: float):
        _check(self._lib.e2d_godunov_unsplit(self._h, int(nStep), float(dt)), "godunov_unsplit", self._h)

    # -- the device-resident time loop
    def step_n(self, n: int, t_end: float, t: float, nstep: int, want_trace: bool = True):
        """Up to n steps of the src/main.cpp loop on the device.
        Returns (t, nstep, dt_trace).  An E2DError raised for a stopped run
        (E2D_ENUMERIC, E2D_ETIMEOUT) carries .t and .nstep: where the loop
        state stands."""
        tt = ctypes.c_double(t)
        ns = ctypes.c_int(nstep)
        trace = np.zeros(max(int(n), 1)) if want_trace else None
        try:
            _check(self._lib.e2d_step_n(self._h, int(n), float(t_end), ctypes.byref(tt), ctypes.byref(ns),
                                        trace.ctypes.data if trace is not None else None),
                   "step_n", self._h)
        except E2DError as e:
            e.t, e.nstep = tt.value, ns.value
            raise
        taken = ns.value - nstep
        return tt.value, ns.value, (trace[:taken] if trace is not None else None)

    def current(self, nstep: int) -> np.ndarray:
        """State after nstep steps (U for even nstep, U2 for odd)."""
        return self.get_state(nstep % 2)

    # -- FP64 audits
    def conservation(self, which: int) -> np.ndarray:
        """FP64 interior sums of (rho, E, mx, my) of state `which`."""
        out = np.zeros(4)
        _check(self._lib.e2d_conservation(self._h, int(which), out.ctypes.data), "conservation", self._h)
        return out

    def l1_diff(self, which: int, other: "HydroRun", other_which: int, var: int = ID):
        """(sum |self - other|, sum |other|) of one variable over the interior,
        accumulated in FP64 on the device."""
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(self._lib.e2d_l1_diff(self._h, int(which), other._h, int(other_which), int(var),
                                     ctypes.byref(a), ctypes.byref(b)), "l1_diff", self._h)
        return a.value, b.value

    # -- Sedov post-processing (src/ComputeRadialProfileFunctor.h:83-165)
    def radial_profile(self, which: int = 0, nbins: int = 0):
        """(distances, mean density, cell count) in nbins rings about the box
        centre over every cell of state `which` (nbins <= 0: [blast] nbins)."""
        n = int(nbins) if nbins > 0 else int(self.params.blast_nbins)
        d, prof = np.zeros(n), np.zeros(n)
        cnt = np.zeros(n, dtype=np.int64)
        _check(self._lib.e2d_radial_profile(self._h, int(which), n, d.ctypes.data, prof.ctypes.data,
                                            cnt.ctypes.data), "radial_profile", self._h)
        return d, prof, cnt

    # -- profiling
    def set_profiling(self, on: bool):
        _check(self._lib.e2d_set_profiling(self._h, int(bool(on))), "set_profiling")

    def kernel_times(self) -> dict:
        n = ctypes.c_int()
        names = (ctypes.c_char_p * 16)()
        ms = (ctypes.c_double * 16)()
        cnt = (ctypes.c_long * 16)()
        _check(self._lib.e2d_kernel_times(self._h, 16, names, ms, cnt, ctypes.byref(n)), "kernel_times")
        return {names[k].decode(): (ms[k], cnt[k]) for k in range(min(n.value, 16))}

    def reset_kernel_times(self):
        self._lib.e2d_reset_kernel_times(self._h)


class Batch:
    """Many independent solves of uneven size (each FP32-compensated or FP64,
    as its parameters say) in one device pool, advanced together
    (e2d_batch_* in include/e2d.h)."""

    def __init__(self, riemann: str = "hllc", pool_bytes: int = 8 << 30, max_instances: int = 1024):
        self._lib = load_library()
        h = ctypes.c_void_p()
        _check(self._lib.e2d_batch_create(RIEMANN[riemann], int(pool_bytes), int(max_instances),
                                          ctypes.byref(h)), "e2d_batch_create")
        self._h = h
        self.riemann = riemann
        self.shapes = {}

    def _ck(self, status, where):
        if status != 0:
            detail = (self._lib.e2d_batch_last_error(self._h) or b"").decode()
            raise E2DError(status, where, detail)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.e2d_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @staticmethod
    def instance_bytes(params: HydroParams) -> int:
        return int(load_library().e2d_batch_instance_bytes(ctypes.byref(params._raw)))

    def free_bytes(self):
        f, l = ctypes.c_size_t(), ctypes.c_size_t()
        self._ck(self._lib.e2d_batch_free_bytes(self._h, ctypes.byref(f), ctypes.byref(l)), "free_bytes")
        return f.value, l.value

    def admit(self, params: HydroParams, t_end: float, u0: np.ndarray | None = None) -> int:
        i = ctypes.c_int()
        ptr = None
        if u0 is not None:
            u0 = np.ascontiguousarray(u0, dtype=np.float64)
            ptr = u0.ctypes.data
        self._ck(self._lib.e2d_batch_admit(self._h, ctypes.byref(params._raw), float(t_end), ptr,
                                           ctypes.byref(i)), "admit")
        self.shapes[i.value] = (4, params.ny + 4, params.nx + 4)
        return i.value

    def run(self, iterations: int) -> int:
        n = ctypes.c_int()
        self._ck(self._lib.e2d_batch_run(self._h, int(iterations), ctypes.byref(n)), "run")
        return n.value

    def query(self, id: int):
        t, ns, a = ctypes.c_double(), ctypes.c_int(), ctypes.c_int()
        self._ck(self._lib.e2d_batch_query(self._h, int(id), ctypes.byref(t), ctypes.byref(ns),
                                           ctypes.byref(a)), "query")
        return t.value, ns.value, bool(a.value)

    def poll(self, id: int):
        """(t, nstep, active, ok) of instance id without raising for a
        stopped solve: ok is False when it hit a non-finite state or a bad dt
        (query's E2D_ENUMERIC) or a device wait of its step gave up
        (E2D_ETIMEOUT), and t, nstep are where it stopped."""
        t, ns, a = ctypes.c_double(), ctypes.c_int(), ctypes.c_int()
        rc = self._lib.e2d_batch_query(self._h, int(id), ctypes.byref(t), ctypes.byref(ns), ctypes.byref(a))
        if rc not in (0, 3, 4):  # E2D_OK, E2D_ENUMERIC, E2D_ETIMEOUT
            self._ck(rc, "query")
        return t.value, ns.value, bool(a.value), rc == 0

    def get_state(self, id: int) -> np.ndarray:
        if id not in self.shapes:
            raise E2DError(1, "get_state", f"instance {id} is not in the batch")  # E2D_EINVAL
        out = np.empty(self.shapes[id], dtype=np.float64)
        self._ck(self._lib.e2d_batch_get_state(self._h, int(id), out.ctypes.data, LAYOUT_LEFT), "get_state")
        return out

    def release(self, id: int):
        self._ck(self._lib.e2d_batch_release(self._h, int(id)), "release")
        self.shapes.pop(id, None)

    def stats(self):
        c, n = ctypes.c_longlong(), ctypes.c_int()
        self._ck(self._lib.e2d_batch_stats(self._h, ctypes.byref(c), ctypes.byref(n)), "stats")
        return c.value, n.value

    def stream(self) -> int:
        s = ctypes.c_void_p()
        self._ck(self._lib.e2d_batch_stream(self._h, ctypes.byref(s)), "stream")
        return s.value or 0

    def set_tuning(self, variant: int = -1, strip_h=None):
        arr = None if strip_h is None else (ctypes.c_int * 3)(*strip_h)
        self._ck(self._lib.e2d_batch_set_tuning(self._h, int(variant), arr), "set_tuning")

    def get_tuning(self):
        v = ctypes.c_int()
        arr = (ctypes.c_int * 3)()
        self._ck(self._lib.e2d_batch_get_tuning(self._h, ctypes.byref(v), arr), "get_tuning")
        return v.value, list(arr)

    def autotune(self, iters_per_trial: int = 2):
        self._ck(self._lib.e2d_batch_autotune(self._h, int(iters_per_trial)), "autotune")


EVAL = {"primitives": (0, 4, 5), "slopes": (1, 20, 8), "trace_xmin": (2, 12, 4), "trace_xmax": (3, 12, 4),
        "trace_ymin": (4, 12, 4), "trace_ymax": (5, 12, 4), "riemann_approx": (6, 8, 4),
        "riemann_hll": (7, 8, 4), "riemann_hllc": (8, 8, 4)}


def write_vtk(params: HydroParams, u: np.ndarray, filename: str, layout: int = LAYOUT_LEFT) -> None:
    """The .vti text writer of HydroRun::saveVTK (src/HydroRun.h:546-607)
    for a host state (ghosts included); no device work."""
    a = np.ascontiguousarray(u, dtype=np.float64)
    if a.size != 4 * params.isize * params.jsize:
        raise ValueError(f"state has {a.size} values, expected {4 * params.isize * params.jsize}")
    _check(load_library().e2d_write_vtk(ctypes.byref(params._raw), a.ctypes.data, int(layout),
                                        os.fsencode(filename)), "write_vtk")


FP64_RATE_NAMES = ("fma", "add", "mul", "div", "sqrt", "max")


def fp64_rates() -> dict:
    """Measured G operations/s of this GPU's FP64 operations (e2d_fp64_rates)."""
    out = np.zeros(6)
    _check(load_library().e2d_fp64_rates(out.ctypes.data), "fp64_rates")
    return dict(zip(FP64_RATE_NAMES, out.tolist()))


def save_npy(path: str, data) -> None:
    """A 1-D double array as an NPY 1.0 file, byte for byte as the
    reference's cnpy::npy_save writes it (src/cnpy/cnpy.h:130-187)."""
    a = np.ascontiguousarray(data, dtype=np.float64).reshape(-1)
    _check(load_library().e2d_save_npy(os.fsencode(path), a.ctypes.data, a.size), "save_npy")


def eval_device(params: HydroParams, what: str, inputs: np.ndarray, dtdx: float = 0.0,
                dtdy: float = 0.0) -> np.ndarray:
    """One building block of the FP64 step (e2d_eval_device) on the device,
    for every row of `inputs` (see include/e2d.h for the row layouts)."""
    code, w_in, w_out = EVAL[what]
    x = np.ascontiguousarray(inputs, dtype=np.float64).reshape(-1, w_in)
    out = np.zeros((len(x), w_out))
    _check(load_library().e2d_eval_device(ctypes.byref(params._raw), code, len(x), x.ctypes.data,
                                          out.ctypes.data, float(dtdx), float(dtdy)), f"eval_device({what})")
    return out
