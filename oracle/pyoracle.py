"""ctypes wrapper of the CPU oracle (oracle/lib/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests, by the smoke check and by the
CPU-baseline leg of bench.py, never by the library.  See the header of
trapbec_oracle.cpp for what it restates and how it is pinned.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from trapbec_gb300.abi import DiagOut, InitArgs, Params, FP64

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, seconds)."""
    if force or not os.path.exists(LIB_PATH) or (
        os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "trapbec_oracle.cpp"))
    ):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(Params)]
        L.orc_destroy.argtypes = [vp]
        L.orc_destroy.restype = None
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads.restype = None
        L.orc_max_threads.restype = C.c_int
        for n in ("orc_set_psi", "orc_get_psi", "orc_get_psi_ghosted", "orc_get_rhs", "orc_velocity",
                  "orc_qpressure"):
            getattr(L, n).argtypes = [vp, vp]
            getattr(L, n).restype = C.c_int
        L.orc_force_vortex.argtypes = [vp, C.c_double, C.c_double, C.c_double]
        L.orc_set_trap.argtypes = [vp, C.POINTER(C.c_double)]
        L.orc_coords.argtypes = [vp] + [C.POINTER(C.c_double)] * 3
        L.orc_apply_damping.argtypes = [vp]
        L.orc_step_rt.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
        L.orc_step_rt_comp.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
        L.orc_step_imag_euler.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
        L.orc_step_imag_rk3.argtypes = [vp, C.c_int, C.c_double, C.POINTER(C.c_int),
                                        C.POINTER(C.c_double)]
        L.orc_set_norm_target.argtypes = [vp, C.c_double]
        L.orc_set_imag_stop.argtypes = [vp, C.c_int, C.c_double]
        L.orc_set_omega.argtypes = [vp, C.c_double]
        L.orc_set_t.argtypes = [vp, C.c_double]
        L.orc_diag.argtypes = [vp, C.POINTER(DiagOut)]
        L.orc_psi_norm_ref.argtypes = [vp]
        L.orc_psi_norm_ref.restype = C.c_double
        L.orc_init_state.argtypes = [vp, C.c_char_p, C.POINTER(InitArgs)]
        L.orc_cell_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L.orc_cell_uniform.restype = C.c_double
        _lib = L
    return _lib


class Oracle:
    """One reference run on the CPU (optionally as nprocx x nprocy ranks)."""

    def __init__(self, params: Params):
        self.p = params.copy()
        self.dtype = np.float64 if params.precision == FP64 else np.float32
        self.cdtype = np.complex128 if params.precision == FP64 else np.complex64
        self.h = lib().orc_create(C.byref(self.p))
        if not self.h:
            raise ValueError("oracle: bad parameters (grid must split evenly)")
        self.shape = (params.nx, params.ny, params.nz)  # C order: x slowest
        self.t = 0.0

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    @staticmethod
    def set_threads(n: int) -> None:
        lib().orc_set_threads(int(n))

    @staticmethod
    def max_threads() -> int:
        return int(lib().orc_max_threads())

    def set_psi(self, psi: np.ndarray) -> None:
        a = np.ascontiguousarray(psi.reshape(self.shape), dtype=self.cdtype)
        assert lib().orc_set_psi(self.h, a.ctypes.data) == 0

    def get_psi(self) -> np.ndarray:
        a = np.empty(self.shape, dtype=self.cdtype)
        assert lib().orc_get_psi(self.h, a.ctypes.data) == 0
        return a

    def get_psi_ghosted(self) -> np.ndarray:
        nx, ny, nz = self.shape
        a = np.empty((nx + 6, ny + 6, nz + 6), dtype=self.cdtype)
        assert lib().orc_get_psi_ghosted(self.h, a.ctypes.data) == 0
        return a

    def get_rhs(self) -> np.ndarray:
        a = np.empty(self.shape, dtype=self.cdtype)
        assert lib().orc_get_rhs(self.h, a.ctypes.data) == 0
        return a

    def force_vortex(self, x0: float, y0: float, direction: float) -> None:
        assert lib().orc_force_vortex(self.h, float(x0), float(y0), float(direction)) == 0

    def velocity(self) -> np.ndarray:
        """get_phase's vel, shape (3, Nx, Ny, Nz)."""
        a = np.empty((3,) + self.shape, dtype=self.dtype)
        assert lib().orc_velocity(self.h, a.ctypes.data) == 0
        return a

    def qpressure(self) -> np.ndarray:
        """get_qpressure's qpressure, shape (3, Nx, Ny, Nz)."""
        a = np.empty((3,) + self.shape, dtype=self.dtype)
        assert lib().orc_qpressure(self.h, a.ctypes.data) == 0
        return a

    def set_trap(self, trap: np.ndarray) -> None:
        a = np.ascontiguousarray(trap.reshape(self.shape), dtype=np.float64)
        assert lib().orc_set_trap(self.h, a.ctypes.data_as(C.POINTER(C.c_double))) == 0

    def coords(self):
        nx, ny, nz = self.shape
        xx, yy, zz = np.empty(nx), np.empty(ny), np.empty(nz)
        P = C.POINTER(C.c_double)
        lib().orc_coords(self.h, xx.ctypes.data_as(P), yy.ctypes.data_as(P), zz.ctypes.data_as(P))
        return xx, yy, zz

    def apply_damping(self) -> None:
        lib().orc_apply_damping(self.h)

    def step_rt(self, n: int) -> float:
        t = C.c_double(self.t)
        lib().orc_step_rt(self.h, int(n), C.byref(t))
        self.t = t.value
        return self.t

    def step_rt_comp(self, n: int) -> float:
        """n RK3 steps with the compensated state (remainders restart at zero on set_psi)."""
        t = C.c_double(self.t)
        lib().orc_step_rt_comp(self.h, int(n), C.byref(t))
        self.t = t.value
        return self.t

    def step_imag_euler(self, n: int) -> float:
        r = C.c_double(0)
        lib().orc_step_imag_euler(self.h, int(n), C.byref(r))
        return r.value

    def step_imag_rk3(self, n: int, tol: float):
        s, r = C.c_int(0), C.c_double(0)
        rc = lib().orc_step_imag_rk3(self.h, int(n), float(tol), C.byref(s), C.byref(r))
        if rc != 0:
            raise RuntimeError(f"oracle imag rk3 failed: {rc}")
        return s.value, r.value

    def set_imag_stop(self, mode: int = 0, energy_scale: float = 0.0) -> None:
        """mode 0: relative stop |dE|/|E| <= tol; 1: absolute |dE| * energy_scale < tol;
        2: absolute per unit norm |dE| / N0 * energy_scale < tol (the trapbec_imag_stop modes)."""
        lib().orc_set_imag_stop(self.h, int(mode), float(energy_scale))

    def set_norm_target(self, n0: float) -> None:
        lib().orc_set_norm_target(self.h, float(n0))

    def set_omega(self, om: float) -> None:
        lib().orc_set_omega(self.h, float(om))

    def set_t(self, t: float) -> None:
        self.t = float(t)
        lib().orc_set_t(self.h, float(t))

    def diag(self) -> dict:
        d = DiagOut()
        lib().orc_diag(self.h, C.byref(d))
        return d.as_dict()

    def psi_norm_ref(self) -> float:
        return float(lib().orc_psi_norm_ref(self.h))

    def init_state(self, name: str, args: InitArgs | None = None) -> None:
        a = args if args is not None else InitArgs()
        rc = lib().orc_init_state(self.h, name.encode(), C.byref(a))
        if rc != 0:
            raise ValueError(f"oracle: unknown initial state {name!r}")


def cell_uniform(seed: int, idx: int, stream: int) -> float:
    return float(lib().orc_cell_uniform(seed, idx, stream))
