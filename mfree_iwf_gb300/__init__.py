"""mfree_iwf_gb300 -- the explicit meshless time step of mfree_iwf on one GB300 (sm_103a).

The compute path is the CUDA library ``libmfree_gb300.so`` behind the C ABI declared
in ``include/mfree_gb300.h``.  This module is a thin host-side mirror of the
reference's set-up interface -- ``body(particles, n, simulation_data, dt, bc)``,
``body::add_action``, ``boundary_conditions::add_boundary_condition``,
``body::set_boundary`` and the step loop of ``main()`` -- over ctypes.  There is no
CPU fallback: if the library is missing, loading it raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import actions
from .actions import *  # noqa: F401,F403  (action ids)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmfree_gb300.so")

METHOD_UL, METHOD_TL, METHOD_TL_WEAK, METHOD_COROT, METHOD_POTENTIAL, METHOD_UL_WEAK = 1, 2, 3, 4, 5, 6
SHAPE_RKPM, SHAPE_ELEMENT = 0, 1  # weak TL shape functions (mf_set_elements)
PREC_FP64_STRICT, PREC_FP64, PREC_MIXED = 0, 1, 2
PRECISIONS = {"fp64_strict": PREC_FP64_STRICT, "fp64": PREC_FP64, "mixed": PREC_MIXED}
BC_PULL = 1       # tensile.cpp:20-42, TL-type bodies
BC_VELOCITY = 2   # tensile.cpp:44-66, UL bodies

STATUS = {
    0: "MF_OK", -1: "MF_ERR_ARG", -2: "MF_ERR_CUDA", -3: "MF_ERR_NBH_OVERFLOW", -4: "MF_ERR_NONFINITE",
    -5: "MF_ERR_TIMEOUT", -6: "MF_ERR_PIPELINE", -7: "MF_ERR_GRID", -8: "MF_ERR_STATE", -9: "MF_ERR_NO_DEVICE",
    -10: "MF_ERR_SINGULAR", -11: "MF_ERR_NO_NEIGHBOR", -12: "MF_ERR_CAPACITY", -13: "MF_ERR_BODY_FAILED",
}

_DP = ctypes.POINTER(ctypes.c_double)
_UP = ctypes.POINTER(ctypes.c_uint32)


class MfConfig(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int32), ("precision", ctypes.c_int32), ("device", ctypes.c_int32),
                ("max_nbh", ctypes.c_uint32), ("nbh_eps", ctypes.c_double), ("nbh_h", ctypes.c_double),
                ("contact", ctypes.c_int32), ("graph", ctypes.c_int32)]


class MfSimData(ctypes.Structure):
    _fields_ = [("nu", ctypes.c_double), ("E", ctypes.c_double), ("rho0", ctypes.c_double),
                ("mghn_wdeltap", ctypes.c_double), ("mghn_corr_exp", ctypes.c_double), ("mghn_eps", ctypes.c_double),
                ("artvisc_alpha", ctypes.c_double), ("artvisc_beta", ctypes.c_double),
                ("artvisc_eta", ctypes.c_double), ("xsph_eps", ctypes.c_double), ("do_smooth", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


_PFIELDS = ("x", "y", "X", "Y", "m", "rho", "h", "quad_weight", "vx", "vy", "Sxx", "Sxy", "Syy")
_SFIELDS = ("x", "y", "vx", "vy", "rho", "Sxx", "Sxy", "Syy", "fcx", "fcy")


class MfParticles(ctypes.Structure):
    _fields_ = [(f, _DP) for f in _PFIELDS]


class MfState(ctypes.Structure):
    _fields_ = [(f, _DP) for f in _SFIELDS]


class MfVtkBody(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("reserved", ctypes.c_uint32)] + [
        (f, _DP) for f in ("x", "y", "h", "rho", "Sxx", "Sxy", "Syy", "vx", "vy")]


DUMP_VTK, DUMP_CHECKPOINT = 0, 1


class MfError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status
        self.name = STATUS.get(status, str(status))


_lib = None


ERR_BODY_FAILED = -13


class BodyFailed(MfError):
    """mf_step with per-body masking: some bodies failed and are frozen; the others
    stepped on.  `failed` holds every body's failure word."""

    def __init__(self, status: int, msg: str, failed: np.ndarray):
        super().__init__(status, msg)
        self.failed = failed


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the CUDA library (raises OSError if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: run mfree_iwf_gb300.build.build() first (there is no CPU fallback)")
    lib = ctypes.CDLL(path)
    C = ctypes
    sig = {
        "mf_create": (C.c_int32, [C.POINTER(MfConfig), C.POINTER(C.c_void_p)]),
        "mf_destroy": (None, [C.c_void_p]),
        "mf_last_error": (C.c_char_p, [C.c_void_p]),
        "mf_status_string": (C.c_char_p, [C.c_int32]),
        "mf_add_body": (C.c_int32, [C.c_void_p, C.POINTER(MfParticles), C.c_uint32, C.POINTER(MfSimData), C.c_double,
                                    C.c_int32, C.POINTER(C.c_int32)]),
        "mf_add_action": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32]),
        "mf_add_boundary_condition": (C.c_int32, [C.c_void_p, C.c_int32, _UP, C.c_uint32, C.c_int32, C.c_double]),
        "mf_set_boundary": (C.c_int32, [C.c_void_p, C.c_int32, _UP, C.c_uint32]),
        "mf_set_gauss_mesh": (C.c_int32, [C.c_void_p, C.c_int32, C.c_uint32, C.c_uint32, C.c_double, C.c_double]),
        "mf_set_stress_points": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_uint32]),
        "mf_set_elements": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32,
                                        C.c_double, C.c_double]),
        "mf_set_gauss_points": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_uint32]),
        "mf_convex_hull": (C.c_int32, [_DP, _DP, C.c_uint32, _UP, _UP]),
        "mf_step": (C.c_int32, [C.c_void_p, C.c_int32]),
        "mf_synchronize": (C.c_int32, [C.c_void_p]),
        "mf_get_state": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(MfState)]),
        "mf_set_state": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(MfParticles)]),
        "mf_get_state_all": (C.c_int32, [C.c_void_p, C.POINTER(MfState)]),
        "mf_set_state_all": (C.c_int32, [C.c_void_p, C.POINTER(MfParticles)]),
        "mf_get_time": (C.c_int32, [C.c_void_p, C.c_int32, _DP]),
        "mf_num_particles": (C.c_int32, [C.c_void_p, C.c_int32, _UP]),
        "mf_get_stress": (C.c_int32, [C.c_void_p, C.c_int32, _DP, _DP, _DP, _DP]),
        "mf_get_state_all_async": (C.c_int32, [C.c_void_p, C.POINTER(MfState)]),
        "mf_set_state_all_async": (C.c_int32, [C.c_void_p, C.POINTER(MfParticles)]),
        "mf_get_failed": (C.c_int32, [C.c_void_p, _UP, C.c_uint32]),
        "mf_get_gauss_state": (C.c_int32, [C.c_void_p, _DP, _DP, _DP, _DP, C.c_uint32, _UP]),
        "mf_get_neighbors": (C.c_int32, [C.c_void_p, C.c_int32, _UP, _UP, C.c_uint64, C.POINTER(C.c_uint64)]),
        "mf_set_timing": (C.c_int32, [C.c_void_p, C.c_int32]),
        "mf_kernel_stats": (C.c_int32, [C.c_void_p, C.c_int32, _DP, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
        "mf_launch_count": (C.c_int32, [C.c_void_p, C.POINTER(C.c_uint64)]),
        "mf_get_stream": (C.c_int32, [C.c_void_p, C.POINTER(C.c_void_p)]),
        "mf_autotune": (C.c_int32, [C.c_void_p, C.c_int32, C.c_char_p, C.c_uint32]),
        "mf_set_monitor": (C.c_int32, [C.c_void_p, C.c_uint32]),
        "mf_set_option": (C.c_int32, [C.c_void_p, C.c_char_p, C.c_int64]),
        "mf_vtk_write": (C.c_int32, [C.c_char_p, C.POINTER(MfVtkBody), C.c_uint32]),
        "mf_dump_async": (C.c_int32, [C.c_void_p, C.c_char_p, C.c_int32]),
        "mf_dump_wait": (C.c_int32, [C.c_void_p]),
        "mf_write_vtk": (C.c_int32, [C.c_void_p, C.c_char_p]),
        "mf_checkpoint_save": (C.c_int32, [C.c_void_p, C.c_char_p]),
        "mf_checkpoint_load": (C.c_int32, [C.c_void_p, C.c_char_p]),
        "mf_get_option": (C.c_int32, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int64)]),
        "mf_get_monitor": (C.c_int32, [C.c_void_p, C.POINTER(C.c_float), _UP]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _dptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(_DP)


def write_vtk_arrays(path: str, bodies: Sequence[Dict[str, np.ndarray]]) -> None:
    """The reference's VTK layout (vtk_writer.h:27-127) from host arrays, one dict per
    body with x, y, h, rho, Sxx, Sxy, Syy, vx, vy (runs on the host only)."""
    lib = load_library()
    keep, arr = [], (MfVtkBody * max(1, len(bodies)))()
    for k, b in enumerate(bodies):
        cols = {f: np.ascontiguousarray(b[f], np.float64) for f in ("x", "y", "h", "rho", "Sxx", "Sxy", "Syy", "vx", "vy")}
        keep.append(cols)
        arr[k] = MfVtkBody(len(cols["x"]), 0, *[_dptr(cols[f]) for f in ("x", "y", "h", "rho", "Sxx", "Sxy", "Syy", "vx", "vy")])
    st = lib.mf_vtk_write(path.encode(), arr, len(bodies))
    if st != 0:
        raise MfError(st, f"mf_vtk_write {path}")


def convex_hull(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """The reference's monotone-chain hull (convex_hull.h:62-95), computed by the library."""
    lib = load_library()
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    out = np.zeros(len(x), np.uint32)
    n = ctypes.c_uint32(0)
    st = lib.mf_convex_hull(_dptr(x), _dptr(y), len(x), out.ctypes.data_as(_UP), ctypes.byref(n))
    if st != 0:
        raise MfError(st, "convex hull")
    return out[: n.value].copy()


@dataclass
class SimData:
    """simulation_data (simulation_data.h:25-99)."""
    nu: float
    E: float
    rho0: float
    mghn_wdeltap: float = 0.0
    mghn_corr_exp: float = 0.0
    mghn_eps: float = 0.0
    artvisc_alpha: float = 0.0
    artvisc_beta: float = 0.0
    artvisc_eta: float = 0.0
    xsph_eps: float = 0.0
    do_smooth: int = 0

    def _c(self) -> MfSimData:
        return MfSimData(self.nu, self.E, self.rho0, self.mghn_wdeltap, self.mghn_corr_exp, self.mghn_eps,
                         self.artvisc_alpha, self.artvisc_beta, self.artvisc_eta, self.xsph_eps, self.do_smooth, 0)


class Simulation:
    """One mf_ctx: a set of bodies stepped together by the reference driver's loop."""

    def __init__(self, method: int = METHOD_UL, precision="fp64_strict", device: int = 0, max_nbh: int = 200,
                 nbh_eps: float = 1e-6, nbh_h: float = 0.0, contact: bool = False, graph: bool = False):
        self._lib = load_library()
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        cfg = MfConfig(method, prec, device, max_nbh, nbh_eps, nbh_h, 1 if contact else 0, 1 if graph else 0)
        h = ctypes.c_void_p()
        st = self._lib.mf_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != 0:
            raise MfError(st, "mf_create")
        self._h = h
        self.method = method
        self.precision = prec
        self._keep: List[object] = []
        self.n_bodies = 0

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mf_destroy(self._h)
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

    def _check(self, st: int, what: str) -> None:
        if st != 0:
            msg = self._lib.mf_last_error(self._h)
            raise MfError(st, f"{what}: {msg.decode() if msg else ''}")

    # -- set-up (body.h:216-233, boundary_conditions.h:32-34)
    def add_body(self, arrays: Dict[str, np.ndarray], sim_data: SimData, dt: float, group: int = 0) -> int:
        n = len(arrays["x"])
        cols = {}
        for f in _PFIELDS:
            a = arrays.get(f)
            cols[f] = None if a is None else np.ascontiguousarray(a, np.float64)
        p = MfParticles(*[_dptr(cols[f]) for f in _PFIELDS])
        bid = ctypes.c_int32(-1)
        sd = sim_data._c()
        self._check(self._lib.mf_add_body(self._h, ctypes.byref(p), n, ctypes.byref(sd), dt, group, ctypes.byref(bid)),
                    "mf_add_body")
        self.n_bodies += 1
        return bid.value

    def add_action(self, body: int, action: int) -> None:
        self._check(self._lib.mf_add_action(self._h, body, int(action)), "mf_add_action")

    def add_boundary_condition(self, body: int, idx: Sequence[int], kind: int, value: float) -> None:
        a = np.ascontiguousarray(idx, np.uint32)
        self._check(self._lib.mf_add_boundary_condition(self._h, body, a.ctypes.data_as(_UP), len(a), kind, value),
                    "mf_add_boundary_condition")

    def set_boundary(self, body: int, idx: Sequence[int]) -> None:
        a = np.ascontiguousarray(idx, np.uint32)
        self._check(self._lib.mf_set_boundary(self._h, body, a.ctypes.data_as(_UP), len(a)), "mf_set_boundary")

    def set_gauss_mesh(self, body: int, ex: int, ey: int, gp_h: float, gp_rho: float) -> None:
        self._check(self._lib.mf_set_gauss_mesh(self._h, body, ex, ey, gp_h, gp_rho), "mf_set_gauss_mesh")

    def set_elements(self, body: int, quads: np.ndarray, order: int, shape: int, gp_h: float, gp_rho: float) -> None:
        """A METHOD_TL_WEAK body's explicit element map (n_elem x 4 body-local particle indices
        ll, lr, tr, tl), Gauss order (1 or 2) and shape kind (SHAPE_RKPM or SHAPE_ELEMENT)."""
        q = np.ascontiguousarray(quads, np.uint32).reshape(-1)
        self._check(self._lib.mf_set_elements(self._h, body, q.ctypes.data_as(_UP), len(q) // 4, int(order), int(shape),
                                              gp_h, gp_rho), "mf_set_elements")

    def set_gauss_points(self, body: int, x, y, h, rho) -> None:
        """The Gauss points' current x, y, h and rho of a METHOD_TL_WEAK body on an explicit
        element map, as the set-up left them."""
        cols = [np.ascontiguousarray(a, np.float64) for a in (x, y, h, rho)]
        self._check(self._lib.mf_set_gauss_points(self._h, body, *[_dptr(a) for a in cols], len(cols[0])),
                    "mf_set_gauss_points")

    def set_stress_points(self, body: int, arrays: Dict[str, np.ndarray]) -> None:
        """The stress points of a METHOD_UL_WEAK body (the particles' 13 fields)."""
        n = len(arrays["x"])
        cols = {f: (None if arrays.get(f) is None else np.ascontiguousarray(arrays[f], np.float64)) for f in _PFIELDS}
        p = MfParticles(*[_dptr(cols[f]) for f in _PFIELDS])
        self._check(self._lib.mf_set_stress_points(self._h, body, ctypes.byref(p), n), "mf_set_stress_points")

    # -- stepping (mfree_iwf.cpp:84-97)
    def step(self, nsteps: int = 1) -> None:
        """Advance every body by nsteps RK4 steps.  With the option "mask_failed" set, a
        body that fails (NaN, neighbour overflow, grid error) is frozen while the others
        step on, and BodyFailed (an MfError) is raised after the steps; failed() names
        the bodies."""
        st = self._lib.mf_step(self._h, int(nsteps))
        if st == ERR_BODY_FAILED:
            raise BodyFailed(st, self._lib.mf_last_error(self._h).decode(), self.failed())
        self._check(st, "mf_step")

    def failed(self) -> np.ndarray:
        """Per-body failure words (0: running; else the ERR bits that failed it)."""
        out = np.zeros(self.n_bodies, np.uint32)
        self._check(self._lib.mf_get_failed(self._h, out.ctypes.data_as(_UP), self.n_bodies), "mf_get_failed")
        return out

    def synchronize(self) -> None:
        """Wait for the queued work; with the option "async_steps" this is where the steps'
        errors surface (BodyFailed for bodies failed under "mask_failed")."""
        st = self._lib.mf_synchronize(self._h)
        if st == ERR_BODY_FAILED:
            raise BodyFailed(st, self._lib.mf_last_error(self._h).decode(), self.failed())
        self._check(st, "mf_synchronize")

    # -- state
    def num_particles(self, body: int) -> int:
        n = ctypes.c_uint32()
        self._check(self._lib.mf_num_particles(self._h, body, ctypes.byref(n)), "mf_num_particles")
        return n.value

    def get_state(self, body: int, fields: Sequence[str] = _SFIELDS) -> Dict[str, np.ndarray]:
        n = self.num_particles(body)
        out = {f: np.empty(n, np.float64) for f in fields}
        s = MfState(*[_dptr(out.get(f)) for f in _SFIELDS])
        self._check(self._lib.mf_get_state(self._h, body, ctypes.byref(s)), "mf_get_state")
        return out

    def get_state_into(self, body: int, out: Dict[str, np.ndarray]) -> None:
        """Device -> caller-owned arrays (contiguous float64, e.g. pinned host memory)."""
        s = MfState(*[_dptr(out.get(f)) for f in _SFIELDS])
        self._check(self._lib.mf_get_state(self._h, body, ctypes.byref(s)), "mf_get_state")

    def set_state(self, body: int, arrays: Dict[str, np.ndarray]) -> None:
        cols = {f: (None if arrays.get(f) is None else np.ascontiguousarray(arrays[f], np.float64)) for f in _PFIELDS}
        p = MfParticles(*[_dptr(cols[f]) for f in _PFIELDS])
        self._check(self._lib.mf_set_state(self._h, body, ctypes.byref(p)), "mf_set_state")

    def get_state_all_into(self, out: Dict[str, np.ndarray]) -> None:
        """Every body's rows (concatenated in body order) -> caller-owned float64 arrays."""
        s = MfState(*[_dptr(out.get(f)) for f in _SFIELDS])
        self._check(self._lib.mf_get_state_all(self._h, ctypes.byref(s)), "mf_get_state_all")

    def set_state_all(self, arrays: Dict[str, np.ndarray]) -> None:
        cols = {f: (None if arrays.get(f) is None else np.ascontiguousarray(arrays[f], np.float64)) for f in _PFIELDS}
        p = MfParticles(*[_dptr(cols[f]) for f in _PFIELDS])
        self._check(self._lib.mf_set_state_all(self._h, ctypes.byref(p)), "mf_set_state_all")

    def get_stress(self, body: int) -> Dict[str, np.ndarray]:
        """The stress the method evaluates at the body's current state: TL (strong form)
        the nominal stress P = J F^-1 sigma, UL the state's S (Pxy = Pyx = Sxy)."""
        n = self.num_particles(body)
        out = {k: np.empty(n, np.float64) for k in ("Pxx", "Pxy", "Pyx", "Pyy")}
        self._check(self._lib.mf_get_stress(self._h, body, *[_dptr(out[k]) for k in ("Pxx", "Pxy", "Pyx", "Pyy")]),
                    "mf_get_stress")
        return out

    def get_gauss_state(self) -> Dict[str, np.ndarray]:
        """The weak TL form's Gauss-point state (rho, Sxx, Sxy, Syy), all bodies."""
        n = ctypes.c_uint32()
        self._check(self._lib.mf_get_gauss_state(self._h, None, None, None, None, 0, ctypes.byref(n)),
                    "mf_get_gauss_state")
        out = {k: np.empty(n.value, np.float64) for k in ("rho", "Sxx", "Sxy", "Syy")}
        self._check(self._lib.mf_get_gauss_state(self._h, *[_dptr(out[k]) for k in ("rho", "Sxx", "Sxy", "Syy")],
                                                 n.value, ctypes.byref(n)), "mf_get_gauss_state")
        return out

    def get_state_all_async_into(self, out: Dict[str, np.ndarray]) -> None:
        """Stream-ordered get_state_all_into: queued behind the steps issued so far; the
        arrays (contiguous float64, pinned for asynchronous copies) hold the state after
        synchronize()."""
        s = MfState(*[_dptr(out.get(f)) for f in _SFIELDS])
        self._check(self._lib.mf_get_state_all_async(self._h, ctypes.byref(s)), "mf_get_state_all_async")

    def set_state_all_async(self, arrays: Dict[str, np.ndarray]) -> None:
        """Stream-ordered set_state_all from contiguous float64 arrays (pinned for
        asynchronous copies; kept alive and unchanged until synchronize()).  Each field
        waits for an earlier get_state_all_async of the same field."""
        for f in _PFIELDS:
            a = arrays.get(f)
            if a is not None and not (a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]):
                raise ValueError(f"{f}: the asynchronous transfer needs contiguous float64 arrays")
        p = MfParticles(*[_dptr(arrays.get(f)) for f in _PFIELDS])
        self._check(self._lib.mf_set_state_all_async(self._h, ctypes.byref(p)), "mf_set_state_all_async")

    def time(self, body: int = 0) -> float:
        t = ctypes.c_double()
        self._check(self._lib.mf_get_time(self._h, body, ctypes.byref(t)), "mf_get_time")
        return t.value

    def neighbor_counts(self, body: int) -> np.ndarray:
        n = self.num_particles(body)
        counts = np.zeros(n, np.uint32)
        tot = ctypes.c_uint64()
        self._check(self._lib.mf_get_neighbors(self._h, body, counts.ctypes.data_as(_UP), None, 0, ctypes.byref(tot)),
                    "mf_get_neighbors")
        return counts

    def neighbors(self, body: int) -> List[np.ndarray]:
        n = self.num_particles(body)
        counts = np.zeros(n, np.uint32)
        tot = ctypes.c_uint64()
        self._check(self._lib.mf_get_neighbors(self._h, body, counts.ctypes.data_as(_UP), None, 0, ctypes.byref(tot)),
                    "mf_get_neighbors")
        idx = np.zeros(max(tot.value, 1), np.uint32)
        self._check(self._lib.mf_get_neighbors(self._h, body, counts.ctypes.data_as(_UP), idx.ctypes.data_as(_UP),
                                               tot.value, ctypes.byref(tot)), "mf_get_neighbors")
        starts = np.concatenate([[0], np.cumsum(counts, dtype=np.int64)])
        return [idx[int(starts[i]):int(starts[i + 1])] for i in range(n)]

    # -- instrumentation
    def set_timing(self, enable: bool) -> None:
        self._check(self._lib.mf_set_timing(self._h, 1 if enable else 0), "mf_set_timing")

    def kernel_stats(self, kind: int):
        ms = ctypes.c_double()
        nl = ctypes.c_uint64()
        rows = ctypes.c_uint64()
        self._check(self._lib.mf_kernel_stats(self._h, kind, ctypes.byref(ms), ctypes.byref(nl), ctypes.byref(rows)),
                    "mf_kernel_stats")
        return ms.value, nl.value, rows.value

    def autotune(self, trial_steps: int = 3) -> str:
        buf = ctypes.create_string_buffer(2048)
        self._check(self._lib.mf_autotune(self._h, int(trial_steps), buf, len(buf)), "mf_autotune")
        return buf.value.decode()

    def set_option(self, key: str, value: int) -> None:
        self._check(self._lib.mf_set_option(self._h, key.encode(), int(value)), "mf_set_option")

    def get_option(self, key: str) -> int:
        v = ctypes.c_int64()
        self._check(self._lib.mf_get_option(self._h, key.encode(), ctypes.byref(v)), "mf_get_option")
        return v.value

    # -- state output (vtk_writer.h) and checkpoints
    def write_vtk(self, path: str) -> None:
        self._check(self._lib.mf_write_vtk(self._h, path.encode()), "mf_write_vtk")

    def dump_async(self, path: str, kind: int = DUMP_VTK) -> None:
        self._check(self._lib.mf_dump_async(self._h, path.encode(), int(kind)), "mf_dump_async")

    def dump_wait(self) -> None:
        self._check(self._lib.mf_dump_wait(self._h), "mf_dump_wait")

    def checkpoint_save(self, path: str) -> None:
        self._check(self._lib.mf_checkpoint_save(self._h, path.encode()), "mf_checkpoint_save")

    def checkpoint_load(self, path: str) -> None:
        self._check(self._lib.mf_checkpoint_load(self._h, path.encode()), "mf_checkpoint_load")

    def set_monitor(self, capacity: int) -> None:
        self._check(self._lib.mf_set_monitor(self._h, int(capacity)), "mf_set_monitor")

    def monitor(self) -> np.ndarray:
        """[rows, bodies, 4]: mean vx, mean vy, max von Mises stress, sum |fc| per step."""
        rows = ctypes.c_uint32()
        self._check(self._lib.mf_get_monitor(self._h, None, ctypes.byref(rows)), "mf_get_monitor")
        out = np.zeros((rows.value, self.n_bodies, 4), np.float32)
        self._check(self._lib.mf_get_monitor(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                             ctypes.byref(rows)), "mf_get_monitor")
        return out

    def launch_count(self) -> int:
        n = ctypes.c_uint64()
        self._check(self._lib.mf_launch_count(self._h, ctypes.byref(n)), "mf_launch_count")
        return n.value

    def stream(self) -> int:
        s = ctypes.c_void_p()
        self._check(self._lib.mf_get_stream(self._h, ctypes.byref(s)), "mf_get_stream")
        return s.value or 0


def from_scenario(sc, precision="fp64_strict", device: int = 0, max_nbh: int = 200, contact: Optional[bool] = None,
                  groups: Optional[Sequence[int]] = None, graph: bool = False) -> Simulation:
    """Build a :class:`Simulation` from a :class:`mfree_iwf_gb300.scenarios.Scenario` (the same
    bodies, constants, action list, boundary conditions and contact boundaries)."""
    sim = Simulation(method=sc.method, precision=precision, device=device, max_nbh=max_nbh, nbh_eps=sc.nbh_eps,
                     nbh_h=sc.nbh_h, contact=bool(sc.contact) if contact is None else contact, graph=graph)
    for k, b in enumerate(sc.bodies):
        p = b.params or {}
        sd = SimData(p.get("nu", sc.nu), p.get("E", sc.E), p.get("rho0", sc.rho0), p.get("wdeltap", sc.wdeltap),
                     sc.corr_exp, sc.mghn_eps, sc.alpha, sc.beta, sc.eta, sc.xsph_eps, sc.do_smooth)
        if groups is not None:
            grp = groups[k]
        elif sc.groups is not None:
            grp = sc.groups[k]
        else:
            grp = 0 if not p else k
        bid = sim.add_body(b.arrays, sd, p.get("dt", sc.dt), group=grp)
        for a in sc.actions:
            sim.add_action(bid, a)
        for bc in b.bcs:
            sim.add_boundary_condition(bid, bc.idx, bc.kind, bc.v)
        if len(b.hull):
            sim.set_boundary(bid, b.hull)
        if sc.method == METHOD_TL_WEAK:
            if b.quads is not None and len(b.quads):
                sim.set_elements(bid, b.quads, b.order, b.shape, sc.gp_h, sc.gp_rho)
                if b.gp is not None:
                    sim.set_gauss_points(bid, b.gp["x"], b.gp["y"], b.gp["h"], b.gp["rho"])
            else:
                sim.set_gauss_mesh(bid, b.ex, b.ey, sc.gp_h, sc.gp_rho)
        if sc.method == METHOD_UL_WEAK:
            if b.quads is not None and len(b.quads):
                sim.set_elements(bid, b.quads, b.order, SHAPE_ELEMENT, 0.0, 0.0)
            sim.set_stress_points(bid, b.gp)
    return sim
