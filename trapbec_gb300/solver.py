"""Host-side mirror of the reference's hot-path operators over libtrapbec.

The reference exposes its time stepping as module procedures on globals
(finite_diff.f90 get_rhs, diagnostic.f90 Psi_norm / Psi_info, the RK3 and
Euler loops of run.f90).  `Solver` gives the same operations, with the same
meaning and units, on one GPU grid.  Arrays are numpy arrays of shape
(Nx, Ny, Nz) in C order, which is the memory order of the Fortran Psi(k,j,i).
There is no CPU fallback: every call goes through the CUDA library.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import check, DiagOut, InitArgs, Params


class Solver:
    def __init__(self, params: Params):
        self.lib = abi.load()
        self.params = params.copy()
        self.ctx = C.c_void_p()
        check(self.lib.trapbec_create(C.byref(self.params), C.byref(self.ctx)), "trapbec_create")
        fp64 = params.precision == abi.FP64
        self.cdtype = np.complex128 if fp64 else np.complex64
        self.rdtype = np.float64 if fp64 else np.float32
        self.shape = (params.nx, params.ny, params.nz)
        self.t = 0.0
        self._held_in, self._held_out = [], []   # host arrays of copies in flight (set/get_psi_async)

    # -- lifetime --------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "ctx", None) and self.ctx.value:
            self.lib.trapbec_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state -----------------------------------------------------------
    def set_psi(self, psi: np.ndarray, layout: int = abi.LAYOUT_INTERIOR) -> None:
        a = np.ascontiguousarray(psi, dtype=self.cdtype)
        want = self.shape if layout == abi.LAYOUT_INTERIOR else tuple(s + 6 for s in self.shape)
        if a.shape != want:
            a = a.reshape(want)
        check(self.lib.trapbec_set_psi(self.ctx, a.ctypes.data, layout), "trapbec_set_psi")

    def get_psi(self, layout: int = abi.LAYOUT_INTERIOR, out: np.ndarray | None = None) -> np.ndarray:
        """psi as a host array; `out` (C-contiguous, the context's complex
        dtype, e.g. a pinned buffer) receives it without another copy."""
        shp = self.shape if layout == abi.LAYOUT_INTERIOR else tuple(s + 6 for s in self.shape)
        if out is None:
            a = np.empty(shp, dtype=self.cdtype)
        else:
            if out.dtype != self.cdtype or out.size != int(np.prod(shp)) or not out.flags["C_CONTIGUOUS"]:
                raise ValueError("get_psi: out must be a C-contiguous array of the context's dtype and size")
            a = out
        check(self.lib.trapbec_get_psi(self.ctx, a.ctypes.data, layout), "trapbec_get_psi")
        return a.reshape(shp)

    # -- overlapped host copies ---------------------------------------------
    def set_psi_async(self, psi: np.ndarray) -> None:
        """Queue `psi` (interior layout; pinned memory lets the copy overlap the steps): it is
        copied up at once and becomes the state at the next step_rt / step_rt_async / step_imag."""
        a = np.ascontiguousarray(psi, dtype=self.cdtype)
        if a.size != int(np.prod(self.shape)):
            raise ValueError("set_psi_async: psi must have the grid's size")
        check(self.lib.trapbec_set_psi_async(self.ctx, a.ctypes.data, abi.LAYOUT_INTERIOR), "trapbec_set_psi_async")
        self._held_in.append(a)

    def get_psi_async(self, out: np.ndarray) -> None:
        """Snapshot the state after the queued steps and copy it into `out` (C-contiguous, the
        context's dtype) in the background; `out` holds it after wait_psi() or synchronize()."""
        if out.dtype != self.cdtype or out.size != int(np.prod(self.shape)) or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("get_psi_async: out must be a C-contiguous array of the context's dtype and size")
        check(self.lib.trapbec_get_psi_async(self.ctx, out.ctypes.data, abi.LAYOUT_INTERIOR), "trapbec_get_psi_async")
        self._held_out.append(out)

    def step_rt_async(self, nsteps: int) -> float:
        """step_rt that returns once the steps are queued; returns the t they reach."""
        t = C.c_double(self.t)
        check(self.lib.trapbec_step_rt_async(self.ctx, int(nsteps), C.byref(t)), "trapbec_step_rt_async")
        self.t = t.value
        return self.t

    def diag_async(self) -> None:
        """Queue diag()'s reduction of the state after the queued steps; diag_wait() returns it."""
        check(self.lib.trapbec_diag_async(self.ctx), "trapbec_diag_async")

    def diag_wait(self) -> dict:
        d = DiagOut()
        check(self.lib.trapbec_diag_wait(self.ctx, C.byref(d)), "trapbec_diag_wait")
        return d.as_dict()

    def wait_psi(self) -> None:
        check(self.lib.trapbec_wait_psi(self.ctx), "trapbec_wait_psi")
        self._held_out.clear()

    def synchronize(self) -> None:
        """Wait for every queued step and copy (reports a timed-out device wait of queued steps)."""
        try:
            check(self.lib.trapbec_synchronize(self.ctx), "trapbec_synchronize")
        finally:
            self._held_in.clear()
            self._held_out.clear()

    def set_trap(self, trap: np.ndarray) -> None:
        a = np.ascontiguousarray(trap.reshape(self.shape), dtype=np.float64)
        check(self.lib.trapbec_set_trap(self.ctx, a.ctypes.data_as(C.POINTER(C.c_double))),
              "trapbec_set_trap")

    def init_state(self, name: str, seed: int = 0, amp: float = 1.0, r_tf2=(0.0, 0.0, 0.0),
                   ring_radius: float = 0.0, core2: float = 0.0, noise_amp: float = 0.0) -> None:
        a = InitArgs()
        a.seed = int(seed)
        a.amp = float(amp)
        for i in range(3):
            a.r_tf2[i] = float(r_tf2[i])
        a.ring_radius = float(ring_radius)
        a.core2 = float(core2)
        a.noise_amp = float(noise_amp)
        check(self.lib.trapbec_init_state(self.ctx, name.encode(), C.byref(a)), "trapbec_init_state")

    # -- the hot path ----------------------------------------------------------
    def get_rhs(self) -> np.ndarray:
        """rhs = get_rhs(psi) (finite_diff.f90:8-136) of the current state."""
        a = np.empty(self.shape, dtype=self.cdtype)
        check(self.lib.trapbec_get_rhs(self.ctx, a.ctypes.data), "trapbec_get_rhs")
        return a

    def step_rt(self, nsteps: int) -> float:
        """nsteps low-storage RK3 steps (run.f90:42-57); returns t."""
        t = C.c_double(self.t)
        check(self.lib.trapbec_step_rt(self.ctx, int(nsteps), C.byref(t)), "trapbec_step_rt")
        self.t = t.value
        return self.t

    def step_imag(self, nsteps: int, variant: int = abi.IMAG_RK3_RENORM, tol: float = 0.0):
        """Imaginary-time relaxation; returns (steps_done, stat)."""
        s, st = C.c_int(0), C.c_double(0)
        check(self.lib.trapbec_step_imag(self.ctx, int(nsteps), int(variant), float(tol),
                                         C.byref(s), C.byref(st)), "trapbec_step_imag")
        return s.value, st.value

    def set_imag_stop(self, mode: int = abi.STOP_REL, energy_scale: float = 1.0) -> None:
        """Stop test of later RK3_RENORM relaxations: abi.STOP_REL (|dE|/|E| <= tol, the default) or
        abi.STOP_ABS (|dE| * energy_scale < tol, energy_scale converting the reference-unit energy
        into the tolerance's unit, e.g. TrapProblem.energy_to_trap(1.0))."""
        check(self.lib.trapbec_set_imag_stop(self.ctx, int(mode), float(energy_scale)), "trapbec_set_imag_stop")

    def diag(self) -> dict:
        d = DiagOut()
        check(self.lib.trapbec_diag(self.ctx, C.byref(d)), "trapbec_diag")
        return d.as_dict()

    def set_wait_limit(self, limit: int = 0, inject: bool = False) -> None:
        """Bounded-wait limit of the tiled kernels in microseconds (0 = default, 2 s); inject = True
        makes every wait run out (test hook of the timeout path)."""
        check(self.lib.trapbec_set_wait_limit(self.ctx, int(limit), int(bool(inject))), "trapbec_set_wait_limit")

    def force_vortex(self, x0: float, y0: float, direction: int) -> None:
        """psi *= pade_density(r) e^{i dir theta} about (x0, y0) (force.f90:33-44)."""
        check(self.lib.trapbec_force_vortex(self.ctx, float(x0), float(y0), float(direction)),
              "trapbec_force_vortex")

    def force_random_points(self, seed: int, draw: int) -> tuple[float, float, float]:
        """force_random_points with draw number `draw` of `seed`; returns (x0, y0, dir)."""
        out = (C.c_double * 3)()
        check(self.lib.trapbec_force_random_points(self.ctx, int(seed), int(draw), out),
              "trapbec_force_random_points")
        return out[0], out[1], out[2]

    def velocity(self) -> np.ndarray:
        """vel of get_phase (diagnostic.f90:27-48), shape (3, Nx, Ny, Nz)."""
        a = np.empty((3,) + self.shape, dtype=self.rdtype)
        check(self.lib.trapbec_get_velocity(self.ctx, a.ctypes.data), "trapbec_get_velocity")
        return a

    def qpressure(self) -> np.ndarray:
        """qpressure of get_qpressure (diagnostic.f90:50-84), shape (3, Nx, Ny, Nz)."""
        a = np.empty((3,) + self.shape, dtype=self.rdtype)
        check(self.lib.trapbec_get_qpressure(self.ctx, a.ctypes.data), "trapbec_get_qpressure")
        return a

    def psi_norm(self) -> float:
        """intPsi2 of Psi_norm (diagnostic.f90:19-25), summed in FP64."""
        return self.diag()["intpsi2"]

    def psi_info(self) -> tuple[float, float, float]:
        """(maxPsi, minPsi, meanPsi) of Psi_info (diagnostic.f90:7-17)."""
        d = self.diag()
        return d["maxpsi"], d["minpsi"], d["meanpsi"]

    # -- controls ----------------------------------------------------------------
    def set_scalar(self, which: int, value: float) -> None:
        check(self.lib.trapbec_set_scalar(self.ctx, int(which), float(value)), "trapbec_set_scalar")
        if which == abi.SCALAR_T:
            self.t = float(value)

    def get_scalar(self, which: int) -> float:
        v = C.c_double(0)
        check(self.lib.trapbec_get_scalar(self.ctx, int(which), C.byref(v)), "trapbec_get_scalar")
        return v.value

    def set_kernel(self, kind: int, tile_z: int = 0, tile_y: int = 0) -> None:
        check(self.lib.trapbec_set_kernel(self.ctx, int(kind), int(tile_z), int(tile_y)),
              "trapbec_set_kernel")

    def set_chunk(self, chunk: int) -> None:
        check(self.lib.trapbec_set_chunk(self.ctx, int(chunk)), "trapbec_set_chunk")

    def tile_shape(self, real_time: bool = True) -> tuple[int, int]:
        """(tile_z, tile_y) of the plain real-time stages (or of every other launch); (0, 0) = per-cell kernel."""
        tz, ty = C.c_int(0), C.c_int(0)
        check(self.lib.trapbec_get_tile_shape(self.ctx, int(bool(real_time)), C.byref(tz), C.byref(ty)),
              "trapbec_get_tile_shape")
        return tz.value, ty.value

    def set_stage_form(self, form: int) -> None:
        """Real-time RK3 form: abi.RK3_THREE_STAGE (default), abi.RK3_DEFERRED (stage 1 stores w1
        only; allocates a second w buffer), abi.RK3_COMPENSATED (FP32: the update keeps its
        rounding remainder in a second array; allocates it) or abi.RK3_PSI_DIFF (no w array:
        each stage recovers the previous stage's w from the two psi arrays)."""
        check(self.lib.trapbec_set_stage_form(self.ctx, int(form)), "trapbec_set_stage_form")

    def stage_form(self) -> int:
        """The form the next step_rt takes."""
        v = C.c_int(0)
        check(self.lib.trapbec_get_stage_form(self.ctx, C.byref(v)), "trapbec_get_stage_form")
        return v.value

    def stage_form_deferred(self) -> bool:
        """True when the next step_rt takes the deferred form."""
        return self.stage_form() == abi.RK3_DEFERRED

    def autotune(self, steps: int = 3) -> dict:
        tz, ty, ch, ms = C.c_int(0), C.c_int(0), C.c_int(0), C.c_double(0)
        check(self.lib.trapbec_autotune(self.ctx, int(steps), C.byref(tz), C.byref(ty), C.byref(ch),
                                        C.byref(ms)), "trapbec_autotune")
        return {"tile_z": tz.value, "tile_y": ty.value, "chunk": ch.value, "ms_per_step": ms.value}

    def launch_count(self) -> int:
        v = C.c_int64(0)
        check(self.lib.trapbec_launch_count(self.ctx, C.byref(v)), "trapbec_launch_count")
        return v.value

    def last_kernel_ms(self) -> float:
        v = C.c_double(0)
        check(self.lib.trapbec_last_kernel_ms(self.ctx, C.byref(v)), "trapbec_last_kernel_ms")
        return v.value

    # -- output layout -------------------------------------------------------------
    def write_var(self, datadir: str, itime: int, shots: int, imaginary: bool = False) -> None:
        check(self.lib.trapbec_write_var(self.ctx, datadir.encode(), int(itime), int(shots),
                                         float(self.t), int(imaginary)), "trapbec_write_var")

    def write_field(self, datadir: str, itime: int, shots: int, which: int) -> None:
        """vel##.dat / qpress##.dat of var_print (output.f90:80-91)."""
        check(self.lib.trapbec_write_field(self.ctx, datadir.encode(), int(itime), int(shots), int(which)),
              "trapbec_write_field")

    def write_restart(self, datadir: str, itime: int) -> None:
        check(self.lib.trapbec_write_restart(self.ctx, datadir.encode(), int(itime), float(self.t)),
              "trapbec_write_restart")

    def read_restart(self, datadir: str) -> int:
        n, t = C.c_int(0), C.c_double(0)
        check(self.lib.trapbec_read_restart(self.ctx, datadir.encode(), C.byref(n), C.byref(t)),
              "trapbec_read_restart")
        self.t = t.value
        return n.value


def parse_cparam(text: str, base: Params | None = None) -> Params:
    """Parse cparam.local text (the reference's compile-time parameters) with
    the library's parser into a Params, starting from `base` or the defaults."""
    lib = abi.load()
    p = base.copy() if base is not None else Params()
    if base is None:
        check(lib.trapbec_params_default(C.byref(p)), "trapbec_params_default")
    err = C.create_string_buffer(256)
    check(lib.trapbec_params_parse(text.encode(), C.byref(p), err, 256), "trapbec_params_parse")
    return p
