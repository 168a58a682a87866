"""ctypes binding of ``libibgpu.so`` (the C ABI in ``include/ib_gpu.h``).

This is the host-side mirror of the reference's Fortran module interface for
the time step: ``Simulation.advance`` is ``timestepper::advance``
(``src/timestepper.F90:18-556``) and the operator functions mirror
``operators_fluid``, ``myfft``, ``fsinterface`` and ``operators_struct``.  Array
arguments are numpy float64 arrays (host memory, staged by the library) or
objects exposing ``data_ptr()`` (CUDA device memory, used in place).

There is no CPU fallback: if the library cannot be loaded, or no GPU is
present, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional, Sequence

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_lib" / "libibgpu.so"

IB_OK = 0
ERRORS = {1: "IB_ERR_ARG", 2: "IB_ERR_CUDA", 3: "IB_ERR_NOMEM", 4: "IB_ERR_GMRES", 5: "IB_ERR_FSI",
          6: "IB_ERR_NONFINITE", 7: "IB_ERR_DOMAIN", 8: "IB_ERR_STATE"}
FIELDS = {"omega": 0, "s": 1, "qx": 2, "qy": 3, "rhs_old": 4, "q0x": 5, "q0y": 6}
VECTORS = {"f": 0, "f_rdst": 1, "xb": 2, "yb": 3, "ub": 4}

# Every symbol include/ib_gpu.h declares (checked by the CPU tests).
EXPORTS = [
    "ib_last_error", "ib_version", "ib_create", "ib_destroy", "ib_synchronize", "ib_advance",
    "ib_get_field", "ib_set_field", "ib_get_vector", "ib_set_vector", "ib_get_forces",
    "ib_get_body_state", "ib_get_counters", "ib_get_dims", "ib_nonlinear", "ib_rot", "ib_curl",
    "ib_coarsify", "ib_get_bc", "ib_apply_bc", "ib_dst", "ib_ctci", "ib_ainv", "ib_fluid_predictor",
    "ib_vort2flux", "ib_reg_prep", "ib_reg", "ib_regT", "ib_redistribute", "ib_schur_apply",
    "ib_schur_apply_fluid", "ib_struct_btimes", "ib_struct_rhs", "ib_struct_dx", "ib_schur_solve",
    "ib_get_stream", "ib_profile", "ib_profile_read", "ib_get_work", "ib_measure_fp64_peak",
    "ib_launch_count", "ib_time_pass", "ib_profile_schur", "ib_ctci_static",
    "ib_schur_matrix", "ib_get_influence_stats", "ib_step_profile", "ib_get_launch_shapes",
    "ib_write_variables", "ib_read_variables", "ib_read_namelist", "ib_read_body", "ib_count_bodies",
    "ib_batch_create", "ib_batch_destroy", "ib_batch_size", "ib_batch_context", "ib_batch_advance",
    "ib_calculate_pressure", "ib_write_pressure", "ib_get_beam_state", "ib_get_step_graph_stats",
    "ib_get_coarse_stats", "ib_get_ring_maps", "ib_set_frame",
    "ib_subdomain_setup", "ib_subdomain_precompute", "ib_write_subdomain_matrix", "ib_read_subdomain_matrix",
    "ib_subdomain_operator", "ib_get_subdomain_stats", "ib_adjoint_forward", "ib_adjoint_backward",
]


class IbError(RuntimeError):
    pass


class IbParams(C.Structure):
    _fields_ = [("m", C.c_int), ("n", C.c_int), ("mgridlev", C.c_int),
                ("dt", C.c_double), ("Re", C.c_double), ("len", C.c_double),
                ("offsetx", C.c_double), ("offsety", C.c_double),
                ("fsi_tol", C.c_double), ("atol", C.c_double), ("rtol", C.c_double),
                ("num_stat", C.c_int), ("motion", C.c_double * 5),
                ("gmres_restart", C.c_int), ("gmres_max_it", C.c_int), ("fsi_max_it", C.c_int),
                ("autotune", C.c_int), ("schur_mode", C.c_int), ("influence_margin", C.c_int)]


class IbRunControl(C.Structure):
    _fields_ = [("istart", C.c_int), ("istop", C.c_int), ("isave", C.c_int), ("irestart", C.c_int),
                ("compute_pressure", C.c_int), ("dimen", C.c_int), ("motion_prescribed", C.c_int),
                ("sub_domain", C.c_int), ("sub_domain_full_rectangular", C.c_int),
                ("sub_domain_precomputed", C.c_int), ("sdxi", C.c_double), ("sdxe", C.c_double),
                ("sdyi", C.c_double), ("sdye", C.c_double), ("delta_sd", C.c_double)]


class IbBody(C.Structure):
    _fields_ = [("npts", C.c_int), ("fam", C.c_int), ("gamma0_deg", C.c_double),
                ("alpha0_deg", C.c_double), ("itheta", C.c_double), ("ktheta", C.c_double),
                ("ctheta", C.c_double), ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)),
                ("nelem", C.c_int)]


_lib = None


def load(path: Optional[os.PathLike] = None):
    """Load the library (building it first if it is missing)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        from . import build as _b
        _b.build()
    lib = C.CDLL(str(p))
    P = C.c_void_p
    D = C.POINTER(C.c_double)
    I = C.POINTER(C.c_int)
    sig = {
        "ib_last_error": ([], C.c_char_p), "ib_version": ([], C.c_int),
        "ib_create": ([C.POINTER(IbParams), C.POINTER(IbBody), C.c_int, C.POINTER(P)], C.c_int),
        "ib_destroy": ([P], C.c_int), "ib_synchronize": ([P], C.c_int), "ib_advance": ([P, I], C.c_int),
        "ib_get_field": ([P, C.c_int, C.c_int, P], C.c_int), "ib_set_field": ([P, C.c_int, C.c_int, P], C.c_int),
        "ib_get_vector": ([P, C.c_int, P], C.c_int), "ib_set_vector": ([P, C.c_int, P], C.c_int),
        "ib_get_forces": ([P, P, P], C.c_int), "ib_get_body_state": ([P, P, P, P], C.c_int),
        "ib_get_counters": ([P, I, I], C.c_int), "ib_get_dims": ([P, I, I, I, I, I], C.c_int),
        "ib_nonlinear": ([P, P, P, P, P, P, P], C.c_int), "ib_rot": ([P, P, P, P], C.c_int),
        "ib_curl": ([P, P, P, P, P], C.c_int), "ib_coarsify": ([P, P, P], C.c_int),
        "ib_get_bc": ([P, P, C.c_double, P], C.c_int), "ib_apply_bc": ([P, P, P, C.c_double], C.c_int),
        "ib_dst": ([P, P, P], C.c_int), "ib_ctci": ([P, P, P], C.c_int), "ib_ainv": ([P, P], C.c_int),
        "ib_fluid_predictor": ([P, C.c_int, P, P, P, P], C.c_int),
        "ib_vort2flux": ([P, P, P, P, P], C.c_int), "ib_reg_prep": ([P, P, P], C.c_int),
        "ib_reg": ([P, P, P, P], C.c_int), "ib_regT": ([P, P, P, P], C.c_int),
        "ib_redistribute": ([P, P, P], C.c_int), "ib_schur_apply": ([P, P, P], C.c_int),
        "ib_schur_apply_fluid": ([P, P, P], C.c_int), "ib_struct_btimes": ([P, P, P], C.c_int),
        "ib_struct_rhs": ([P, P], C.c_int), "ib_struct_dx": ([P, P, P], C.c_int),
        "ib_schur_solve": ([P, P, P, I], C.c_int),
        "ib_get_stream": ([P, C.POINTER(P)], C.c_int), "ib_profile": ([P, C.c_int], C.c_int),
        "ib_profile_read": ([P, C.c_int, I, D, D], C.c_int),
        "ib_get_work": ([P, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)], C.c_int),
        "ib_measure_fp64_peak": ([D], C.c_int),
        "ib_launch_count": ([], C.c_longlong),
        "ib_time_pass": ([P, C.c_int, C.c_int, D], C.c_int),
        "ib_profile_schur": ([P, C.c_int, D], C.c_int),
        "ib_ctci_static": ([C.c_int, C.c_int, P, P, P], C.c_int),
        "ib_schur_matrix": ([P, P, C.POINTER(C.c_int)], C.c_int),
        "ib_step_profile": ([P, C.c_int, D, C.POINTER(C.c_longlong)], C.c_int),
        "ib_get_influence_stats": ([P, C.POINTER(C.c_longlong), D], C.c_int),
        "ib_get_launch_shapes": ([P, I], C.c_int),
        "ib_write_variables": ([P, C.c_char_p], C.c_int),
        "ib_read_variables": ([P, C.c_char_p, C.c_int], C.c_int),
        "ib_read_namelist": ([C.c_char_p, C.POINTER(IbParams), C.POINTER(IbRunControl)], C.c_int),
        "ib_read_body": ([C.c_char_p, C.POINTER(IbBody), D, D, C.c_int], C.c_int),
        "ib_count_bodies": ([C.c_char_p, I], C.c_int),
        "ib_batch_create": ([C.POINTER(IbParams), C.POINTER(IbBody), I, C.c_int, C.POINTER(P)], C.c_int),
        "ib_batch_destroy": ([P], C.c_int), "ib_batch_size": ([P, I], C.c_int),
        "ib_batch_context": ([P, C.c_int, C.POINTER(P)], C.c_int),
        "ib_batch_advance": ([P, I], C.c_int),
        "ib_calculate_pressure": ([P, P], C.c_int), "ib_write_pressure": ([P, C.c_char_p], C.c_int),
        "ib_get_beam_state": ([P, P, P, P], C.c_int),
        "ib_get_step_graph_stats": ([P, C.POINTER(C.c_longlong)], C.c_int),
        "ib_get_coarse_stats": ([P, C.POINTER(C.c_longlong), C.POINTER(C.c_double)], C.c_int),
        "ib_get_ring_maps": ([P, C.POINTER(C.c_longlong), C.POINTER(C.c_double)], C.c_int),
        "ib_set_frame": ([P, P], C.c_int),
        "ib_subdomain_setup": ([P, C.c_int] + [C.c_double] * 5, C.c_int),
        "ib_subdomain_precompute": ([P], C.c_int),
        "ib_write_subdomain_matrix": ([P, C.c_char_p], C.c_int),
        "ib_read_subdomain_matrix": ([P, C.c_char_p], C.c_int),
        "ib_subdomain_operator": ([P, P], C.c_int),
        "ib_get_subdomain_stats": ([P, C.POINTER(C.c_longlong), D], C.c_int),
        "ib_adjoint_forward": ([P, C.c_int, C.c_int, P, P], C.c_int),
        "ib_adjoint_backward": ([P, P, P], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def _check(rc: int, what: str = ""):
    if rc != IB_OK:
        msg = load().ib_last_error().decode(errors="replace")
        raise IbError(f"{what}: {ERRORS.get(rc, rc)}: {msg}")


def _ptr(a):
    """Pointer of a float64 numpy array (host) or a CUDA tensor (device)."""
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]):
        raise TypeError("arrays must be C-contiguous float64 numpy arrays or CUDA tensors")
    return C.c_void_p(a.ctypes.data)


def launch_count() -> int:
    """Kernels launched by libibgpu.so since it was loaded."""
    return int(load().ib_launch_count())


def ctci_static(m: int, n: int, vort_ptr: int, s_ptr: int, stream_ptr: int = 0) -> None:
    """Context-free Poisson solve on device arrays (raw device addresses), allocating nothing.

    Runs asynchronously on the given CUDA stream (0: the default stream); the grid must fit
    the library's 16 MiB static scratch, and calls that overlap on the GPU race on it."""
    _check(load().ib_ctci_static(m, n, C.c_void_p(vort_ptr), C.c_void_p(s_ptr), C.c_void_p(stream_ptr)),
           "ib_ctci_static")


def measure_fp64_peak() -> float:
    """FP64 FMA throughput of the current GPU in TFLOP/s."""
    t = C.c_double()
    _check(load().ib_measure_fp64_peak(C.byref(t)), "ib_measure_fp64_peak")
    return t.value


@dataclass
class Body:
    """One ``input/body.NNN.inp`` (grid.F90:252-288): fam 1 rigid, 2 torsional, 3 Euler-Bernoulli
    beam (itheta = mass per unit length, ktheta = EI, nelem elements; 0: (npts - 1) / 2)."""
    x: np.ndarray
    y: np.ndarray
    fam: int = 1
    gamma0_deg: float = 0.0
    alpha0_deg: float = 0.0
    itheta: float = 0.0
    ktheta: float = 0.0
    ctheta: float = 0.0
    nelem: int = 0

    @property
    def npts(self):
        return len(self.x)


@dataclass
class Params:
    """Namelist ``read_parameters`` (parameters.F90:55-59)."""
    m: int
    n: int
    mgridlev: int
    dt: float
    Re: float
    len: float
    offsetx: float
    offsety: float
    fsi_tol: float = 1e-10
    atol: float = 1e-10
    rtol: float = 1e-10
    num_stat: bool = False
    motion: tuple = (-1.0, 0.0, 0.0, 0.0, 0.0)
    gmres_restart: int = 30
    gmres_max_it: int = 10000
    fsi_max_it: int = 1000
    autotune: bool = True
    schur_mode: int = 0          # 0 influence matrix + one-kernel GMRES, 1 matrix-free, 2 influence + graph GMRES
    influence_margin: int = 0    # band slack in vertices (0: 8)

    def to_c(self) -> IbParams:
        p = IbParams()
        for k in ("m", "n", "mgridlev", "gmres_restart", "gmres_max_it", "fsi_max_it"):
            setattr(p, k, int(getattr(self, k)))
        for k in ("dt", "Re", "len", "offsetx", "offsety", "fsi_tol", "atol", "rtol"):
            setattr(p, k, float(getattr(self, k)))
        p.num_stat = int(bool(self.num_stat))
        p.autotune = int(bool(self.autotune))
        p.schur_mode = int(self.schur_mode)
        p.influence_margin = int(self.influence_margin)
        for i in range(5):
            p.motion[i] = float(self.motion[i])
        return p


def _c_bodies(bodies: Sequence[Body], keep: list):
    """A ctypes IbBody array of the bodies (their coordinate arrays appended to keep)."""
    cb = (IbBody * max(1, len(bodies)))()
    for i, b in enumerate(bodies):
        x = np.ascontiguousarray(b.x, dtype=np.float64)
        y = np.ascontiguousarray(b.y, dtype=np.float64)
        keep += [x, y]
        cb[i].npts = len(x)
        cb[i].fam = int(b.fam)
        cb[i].gamma0_deg = float(b.gamma0_deg)
        cb[i].alpha0_deg = float(b.alpha0_deg)
        cb[i].itheta = float(b.itheta)
        cb[i].ktheta = float(b.ktheta)
        cb[i].ctheta = float(b.ctheta)
        cb[i].x = x.ctypes.data_as(C.POINTER(C.c_double))
        cb[i].y = y.ctypes.data_as(C.POINTER(C.c_double))
        cb[i].nelem = int(getattr(b, "nelem", 0))
    return cb


class Simulation:
    """One device-resident simulation (an ``IbCtx``)."""

    def __init__(self, params: Params, bodies: Sequence[Body] = (), _handle=None):
        self.lib = load()
        self.params = params
        self._keep = []
        self._owned = _handle is None
        if _handle is None:
            cb = _c_bodies(bodies, self._keep)
            h = C.c_void_p()
            cp = params.to_c()
            _check(self.lib.ib_create(C.byref(cp), cb, len(bodies), C.byref(h)), "ib_create")
        else:
            h = _handle
        self.h = h
        self.nbody = len(bodies)
        self.ntors = sum(1 for b in bodies if b.fam == 2)
        self.beam_dofs = sum(2 * (b.nelem or (b.npts - 1) // 2) for b in bodies if b.fam == 3)
        nf, nbc, ns, nu, nv = (C.c_int() for _ in range(5))
        _check(self.lib.ib_get_dims(self.h, C.byref(nf), C.byref(nbc), C.byref(ns), C.byref(nu), C.byref(nv)))
        self.nf, self.nbc, self.ns, self.nu, self.nv = nf.value, nbc.value, ns.value, nu.value, nv.value
        m, n = params.m, params.n
        self.shapes = {"omega": (n - 1, m - 1), "s": (n - 1, m - 1), "rhs_old": (n - 1, m - 1),
                       "qx": (n, m + 1), "q0x": (n, m + 1), "qy": (n + 1, m), "q0y": (n + 1, m)}

    def close(self):
        if getattr(self, "h", None):
            if self._owned:
                self.lib.ib_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- stepping and state
    def advance(self) -> int:
        it = C.c_int()
        _check(self.lib.ib_advance(self.h, C.byref(it)), "ib_advance")
        return it.value

    def pressure(self) -> list:
        """calculate_pressure (operators_pressure.F90:110-437): the pressure coefficient at the
        cell centres of every level, a list of (n, m) arrays."""
        L, m, n = self.params.mgridlev, self.params.m, self.params.n
        out = np.empty((L, n, m))
        _check(self.lib.ib_calculate_pressure(self.h, _ptr(out)), "ib_calculate_pressure")
        return list(out)

    def write_pressure(self, path) -> None:
        _check(self.lib.ib_write_pressure(self.h, os.fsencode(path)), "ib_write_pressure")

    def write_variables(self, path) -> None:
        """write_variables (variables.F90:709-803): the reference's restart file at path."""
        _check(self.lib.ib_write_variables(self.h, os.fsencode(path)), "ib_write_variables")

    def read_variables(self, path, itime: int) -> None:
        """read_variables (variables.F90:807-913): restore the state; the next step is itime + 1."""
        _check(self.lib.ib_read_variables(self.h, os.fsencode(path), int(itime)), "ib_read_variables")

    def get_field(self, name: str, level: int = 0) -> np.ndarray:
        out = np.empty(self.shapes[name])
        _check(self.lib.ib_get_field(self.h, FIELDS[name], level, _ptr(out)), "ib_get_field")
        return out

    def set_frame(self, u: float, v: float, w: float) -> None:
        """The frame's velocity (u, v) and angular velocity w for the steps that follow (the
        frame fluxes q0 of every level formed on the device)."""
        a = np.array([u, v, w], dtype=np.float64)
        _check(self.lib.ib_set_frame(self.h, _ptr(a)), "ib_set_frame")

    def set_field(self, name: str, level: int, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64) if not hasattr(arr, "data_ptr") else arr
        _check(self.lib.ib_set_field(self.h, FIELDS[name], level, _ptr(a)), "ib_set_field")

    def get_vector(self, name: str) -> np.ndarray:
        out = np.empty(self.nf)
        _check(self.lib.ib_get_vector(self.h, VECTORS[name], _ptr(out)), "ib_get_vector")
        return out

    def set_vector(self, name: str, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        _check(self.lib.ib_set_vector(self.h, VECTORS[name], _ptr(a)), "ib_set_vector")

    def forces(self):
        cx = np.empty(max(1, self.nbody)); cy = np.empty(max(1, self.nbody))
        _check(self.lib.ib_get_forces(self.h, _ptr(cx), _ptr(cy)), "ib_get_forces")
        return cx[:self.nbody], cy[:self.nbody]

    def body_state(self):
        n = max(1, self.ntors)
        a, b, c = np.zeros(n), np.zeros(n), np.zeros(n)
        _check(self.lib.ib_get_body_state(self.h, _ptr(a), _ptr(b), _ptr(c)), "ib_get_body_state")
        return a[:self.ntors], b[:self.ntors], c[:self.ntors]

    def beam_state(self):
        """DOFs (w, dw/ds at the free nodes) of the beams, their rates and accelerations."""
        n = max(1, self.beam_dofs)
        a, b, c = np.zeros(n), np.zeros(n), np.zeros(n)
        _check(self.lib.ib_get_beam_state(self.h, _ptr(a), _ptr(b), _ptr(c)), "ib_get_beam_state")
        return a[:self.beam_dofs], b[:self.beam_dofs], c[:self.beam_dofs]

    def counters(self):
        k, f = C.c_int(), C.c_int()
        _check(self.lib.ib_get_counters(self.h, C.byref(k), C.byref(f)))
        return k.value, f.value

    def stream(self) -> int:
        s = C.c_void_p()
        _check(self.lib.ib_get_stream(self.h, C.byref(s)), "ib_get_stream")
        return s.value or 0

    def time_pass(self, kind: int, reps: int = 20) -> float:
        """Average device ms of one full x pass (0) or tridiagonal solve (1) timed alone."""
        ms = C.c_double()
        _check(self.lib.ib_time_pass(self.h, kind, reps, C.byref(ms)), "ib_time_pass")
        return ms.value

    SCHUR_STAGES = ["reg+rot", "ainv", "coarsify", "coarse levels", "finest forward", "finest solve",
                    "finest inverse rows", "E curl + B"]

    def profile_schur(self, reps: int = 20) -> dict:
        """Average device us per Schur application of each of its stages."""
        out = (C.c_double * 8)()
        _check(self.lib.ib_profile_schur(self.h, reps, out), "ib_profile_schur")
        return {n: 1e3 * out[i] / reps for i, n in enumerate(self.SCHUR_STAGES)}

    def schur_matrix(self):
        """Assembled fluid Schur matrix (nf x nf) from the influence matrix, or None when the
        solver falls back to the matrix-free operator at the current positions."""
        S = np.zeros((self.nf, self.nf))
        st = C.c_int(0)
        _check(self.lib.ib_schur_matrix(self.h, _ptr(S), C.byref(st)), "ib_schur_matrix")
        return S if st.value == 0 else None

    STEP_PHASES = ["predictor", "vort2flux", "fsi rhs", "schur assembly", "gmres", "fsi update", "correction",
                   "fsi device loop"]

    def step_profile(self, mode: int) -> dict:
        """mode 1 start (FSI iterations from the host, phase by phase), 3 start (device FSI loop
        kept, timed as one phase), 0 stop, 2 read: average device us per step of each phase."""
        ms = (C.c_double * 8)()
        n = C.c_longlong(0)
        _check(self.lib.ib_step_profile(self.h, mode, ms, C.byref(n)), "ib_step_profile")
        return {k: (1e3 * ms[i] / n.value if n.value else 0.0) for i, k in enumerate(self.STEP_PHASES)}

    def launch_shapes(self) -> dict:
        """The launch shapes the context runs with (tuned at creation when autotune is set)."""
        v = (C.c_int * 13)()
        _check(self.lib.ib_get_launch_shapes(self.h, v), "ib_get_launch_shapes")
        names = ["x_one_level", "x_few_rows", "x_all_levels", "y"]
        out = {n: {"lines_per_cta": v[3 * i], "threads": v[3 * i + 1], "one_warp_scan": v[3 * i + 2]}
               for i, n in enumerate(names)}
        out["tridiagonal_modes_per_cta"] = v[12]
        return out

    def influence_stats(self) -> dict:
        counts = (C.c_longlong * 5)()
        ms = C.c_double()
        _check(self.lib.ib_get_influence_stats(self.h, counts, C.byref(ms)), "ib_get_influence_stats")
        return {"builds": counts[0], "columns": counts[1], "assemblies": counts[2], "fallbacks": counts[3],
                "band_vertices": counts[4], "build_ms": ms.value}

    # ---- the sub-domain precomputed-Schur method (sub_domain = T)
    def subdomain_setup(self, sdxi: float, sdxe: float, sdyi: float, sdye: float, delta_sd: float,
                        full_rectangular: bool = True) -> None:
        """Switches the context to the sub-domain method (before its first step)."""
        _check(self.lib.ib_subdomain_setup(self.h, int(bool(full_rectangular)), C.c_double(sdxi),
                                           C.c_double(sdxe), C.c_double(sdyi), C.c_double(sdye),
                                           C.c_double(delta_sd)), "ib_subdomain_setup")

    def subdomain_precompute(self) -> None:
        _check(self.lib.ib_subdomain_precompute(self.h), "ib_subdomain_precompute")

    def write_subdomain_matrix(self, path) -> None:
        _check(self.lib.ib_write_subdomain_matrix(self.h, str(path).encode()), "ib_write_subdomain_matrix")

    def read_subdomain_matrix(self, path) -> None:
        _check(self.lib.ib_read_subdomain_matrix(self.h, str(path).encode()), "ib_read_subdomain_matrix")

    def subdomain_operator(self) -> np.ndarray:
        """body + P B^T P^T at the current positions (nf x nf)."""
        out = np.zeros((self.nf, self.nf))
        _check(self.lib.ib_subdomain_operator(self.h, _ptr(out)), "ib_subdomain_operator")
        return out

    def subdomain_stats(self) -> dict:
        counts = (C.c_longlong * 4)()
        ms = C.c_double()
        _check(self.lib.ib_get_subdomain_stats(self.h, counts, C.byref(ms)), "ib_get_subdomain_stats")
        return {"unknowns": counts[0], "candidates": counts[1], "kept": counts[2], "columns": counts[3],
                "precompute_ms": ms.value}

    # ---- the discrete adjoint (stationary rigid bodies, num_stat, moving frame)
    def adjoint_forward(self, frames, K: int = 20) -> np.ndarray:
        """Advances len(frames) steps with per-step frame (u, v, W); returns the force
        coefficients (nsteps, nbody, 2), keeping checkpoints for adjoint_backward."""
        fr = np.ascontiguousarray(frames, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((fr.shape[0], max(1, self.nbody), 2))
        _check(self.lib.ib_adjoint_forward(self.h, fr.shape[0], int(K), _ptr(fr), _ptr(out)), "ib_adjoint_forward")
        return out[:, :self.nbody]

    def adjoint_backward(self, dforces) -> np.ndarray:
        """dJ/dframes (nsteps, 3) for J = sum(dforces * forces) of the last adjoint_forward."""
        d = np.ascontiguousarray(dforces, dtype=np.float64)
        out = np.zeros((d.shape[0], 3))
        _check(self.lib.ib_adjoint_backward(self.h, _ptr(d), _ptr(out)), "ib_adjoint_backward")
        return out

    def step_graph_stats(self) -> dict:
        """How the steps ran: as one graph, of those with the FSI loop finished from the host,
        and phase by phase."""
        counts = (C.c_longlong * 3)()
        _check(self.lib.ib_get_step_graph_stats(self.h, counts), "ib_get_step_graph_stats")
        return {"graph": counts[0], "gate_closed": counts[1], "phased": counts[2]}

    def coarse_stats(self) -> dict:
        """The coarse levels' responses behind the band build and the sub-domain precompute:
        level solves run, responses held, their bytes, whether enabled, host milliseconds."""
        counts = (C.c_longlong * 4)()
        ms = C.c_double()
        _check(self.lib.ib_get_coarse_stats(self.h, counts, C.byref(ms)), "ib_get_coarse_stats")
        return {"solves": counts[0], "held": counts[1], "bytes": counts[2], "enabled": bool(counts[3]),
                "ms": ms.value}

    def ring_maps(self) -> dict:
        """The ring maps of the predictor's and vort2flux's coarse-to-fine recursions: whether in
        use, their bytes, host milliseconds of their precomputation."""
        counts = (C.c_longlong * 2)()
        ms = C.c_double()
        _check(self.lib.ib_get_ring_maps(self.h, counts, C.byref(ms)), "ib_get_ring_maps")
        return {"on": bool(counts[0]), "bytes": counts[1], "ms": ms.value}

    def profile(self, enable: bool):
        _check(self.lib.ib_profile(self.h, int(bool(enable))), "ib_profile")

    def profile_read(self, kind: int):
        n, t, b = C.c_int(), C.c_double(), C.c_double()
        _check(self.lib.ib_profile_read(self.h, kind, C.byref(n), C.byref(t), C.byref(b)), "ib_profile_read")
        return n.value, t.value, b.value

    def work(self):
        mv = C.c_longlong()
        passes = (C.c_longlong * 4)()
        _check(self.lib.ib_get_work(self.h, C.byref(mv), passes), "ib_get_work")
        return mv.value, list(passes)

    def synchronize(self):
        _check(self.lib.ib_synchronize(self.h), "ib_synchronize")

    # ---- operators (mirror the Fortran routines)
    def _o(self, shape):
        return np.zeros(shape)

    def nonlinear(self, omega, qx, qy, bc):
        nlx = self._o(self.shapes["qx"]); nly = self._o(self.shapes["qy"])
        _check(self.lib.ib_nonlinear(self.h, _ptr(omega), _ptr(qx), _ptr(qy), _ptr(bc), _ptr(nlx), _ptr(nly)),
               "ib_nonlinear")
        return nlx, nly

    def rot(self, hx, hy):
        v = self._o(self.shapes["omega"])
        _check(self.lib.ib_rot(self.h, _ptr(hx), _ptr(hy), _ptr(v)), "ib_rot")
        return v

    def curl(self, s, sbc):
        qx = self._o(self.shapes["qx"]); qy = self._o(self.shapes["qy"])
        _check(self.lib.ib_curl(self.h, _ptr(s), _ptr(sbc), _ptr(qx), _ptr(qy)), "ib_curl")
        return qx, qy

    def coarsify(self, fine, coarse):
        out = np.array(coarse, dtype=np.float64, copy=True)
        _check(self.lib.ib_coarsify(self.h, _ptr(fine), _ptr(out)), "ib_coarsify")
        return out

    def get_bc(self, s, fac):
        ring = np.zeros(self.nbc)
        _check(self.lib.ib_get_bc(self.h, _ptr(s), C.c_double(fac), _ptr(ring)), "ib_get_bc")
        return ring

    def apply_bc(self, vort, ring, fac):
        out = np.array(vort, dtype=np.float64, copy=True)
        _check(self.lib.ib_apply_bc(self.h, _ptr(out), _ptr(ring), C.c_double(fac)), "ib_apply_bc")
        return out

    def dst(self, x):
        out = self._o(self.shapes["omega"])
        _check(self.lib.ib_dst(self.h, _ptr(np.ascontiguousarray(x)), _ptr(out)), "ib_dst")
        return out

    def ctci(self, x):
        out = self._o(self.shapes["omega"])
        _check(self.lib.ib_ctci(self.h, _ptr(np.ascontiguousarray(x)), _ptr(out)), "ib_ctci")
        return out

    def ainv(self, x):
        out = np.array(x, dtype=np.float64, copy=True)
        _check(self.lib.ib_ainv(self.h, _ptr(out)), "ib_ainv")
        return out

    def fluid_predictor(self, level, omega, rhs, rhs_old, rhsbc):
        out = np.array(omega, dtype=np.float64, copy=True)
        _check(self.lib.ib_fluid_predictor(self.h, level, _ptr(out), _ptr(rhs), _ptr(rhs_old), _ptr(rhsbc)),
               "ib_fluid_predictor")
        return out

    def vort2flux(self, omega_levels):
        L = self.params.mgridlev
        w = np.ascontiguousarray(np.stack(omega_levels), dtype=np.float64).copy()
        s = np.zeros_like(w)
        qx = np.zeros((L,) + self.shapes["qx"]); qy = np.zeros((L,) + self.shapes["qy"])
        _check(self.lib.ib_vort2flux(self.h, _ptr(w), _ptr(s), _ptr(qx), _ptr(qy)), "ib_vort2flux")
        return list(w), list(s), list(qx), list(qy)

    def reg_prep(self, xb, yb):
        _check(self.lib.ib_reg_prep(self.h, _ptr(np.ascontiguousarray(xb, dtype=np.float64)),
                                    _ptr(np.ascontiguousarray(yb, dtype=np.float64))), "ib_reg_prep")

    def reg(self, h0):
        hx = self._o(self.shapes["qx"]); hy = self._o(self.shapes["qy"])
        _check(self.lib.ib_reg(self.h, _ptr(np.ascontiguousarray(h0, dtype=np.float64)), _ptr(hx), _ptr(hy)),
               "ib_reg")
        return hx, hy

    def regT(self, hx, hy, h0=None):
        out = np.zeros(self.nf) if h0 is None else np.array(h0, dtype=np.float64, copy=True)
        _check(self.lib.ib_regT(self.h, _ptr(hx), _ptr(hy), _ptr(out)), "ib_regT")
        return out

    def redistribute(self, f):
        out = np.zeros(self.nf)
        _check(self.lib.ib_redistribute(self.h, _ptr(np.ascontiguousarray(f, dtype=np.float64)), _ptr(out)),
               "ib_redistribute")
        return out

    def schur_apply(self, x, with_b=True):
        out = np.zeros(self.nf)
        fn = self.lib.ib_schur_apply if with_b else self.lib.ib_schur_apply_fluid
        _check(fn(self.h, _ptr(np.ascontiguousarray(x, dtype=np.float64)), _ptr(out)), "ib_schur_apply")
        return out

    def struct_btimes(self, x):
        out = np.zeros(self.nf)
        _check(self.lib.ib_struct_btimes(self.h, _ptr(np.ascontiguousarray(x, dtype=np.float64)), _ptr(out)))
        return out

    def struct_rhs(self):
        out = np.zeros(self.nf)
        _check(self.lib.ib_struct_rhs(self.h, _ptr(out)), "ib_struct_rhs")
        return out

    def struct_dx(self, f) -> float:
        """compute_dx (operators_struct.F90:402-505): hinge angles and positions from force f;
        returns the FSI error max |dtheta|."""
        err = C.c_double()
        _check(self.lib.ib_struct_dx(self.h, _ptr(np.ascontiguousarray(f, dtype=np.float64)), C.byref(err)),
               "ib_struct_dx")
        return err.value

    def schur_solve(self, rhs, f0):
        f = np.array(f0, dtype=np.float64, copy=True)
        its = C.c_int()
        _check(self.lib.ib_schur_solve(self.h, _ptr(np.ascontiguousarray(rhs, dtype=np.float64)), _ptr(f),
                                       C.byref(its)), "ib_schur_solve")
        return f, its.value



class Batch:
    """Independent simulations advanced together (``ib_batch_*``): each keeps its own grid,
    bodies, device memory and stream, and a batch step queues every simulation's work before
    waiting on any.  ``sims[i]`` is a Simulation view of simulation i (owned by the batch)."""

    def __init__(self, runs: Sequence[tuple]):
        self.lib = load()
        self._keep = []
        n = len(runs)
        cps = (IbParams * n)()
        all_bodies = [b for _, bodies in runs for b in bodies]
        cb = _c_bodies(all_bodies, self._keep)
        nb = (C.c_int * n)(*[len(bodies) for _, bodies in runs])
        for i, (p, _) in enumerate(runs):
            cps[i] = p.to_c()
        h = C.c_void_p()
        _check(self.lib.ib_batch_create(cps, cb, nb, n, C.byref(h)), "ib_batch_create")
        self.h = h
        self.status = (C.c_int * n)()
        self.sims = []
        for i, (p, bodies) in enumerate(runs):
            ch = C.c_void_p()
            _check(self.lib.ib_batch_context(self.h, i, C.byref(ch)), "ib_batch_context")
            self.sims.append(Simulation(p, bodies, _handle=ch))

    def advance(self, check: bool = True) -> list:
        """One step of every simulation; returns the per-simulation status codes."""
        rc = self.lib.ib_batch_advance(self.h, self.status)
        if check:
            _check(rc, "ib_batch_advance")
        return list(self.status)

    def close(self):
        if getattr(self, "h", None):
            for s in self.sims:
                s.h = None
            self.lib.ib_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
