"""Batched imaginary-time ground states over libtrapbec (trapbec_batch_*).

Many independent grids (own size, box, trap, rotation and step) are relaxed
together by the RK3 imaginary-time loop with FP64 renormalisation and an
energy-change stop (relative by default, absolute per set_imag_stop); each RK3
stage is one persistent launch over the work of all unconverged grids and the
step loop is replayed from a CUDA graph.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import check, InitArgs, Params


class BatchSolver:
    def __init__(self, params: list[Params]):
        self.lib = abi.load()
        self.n = len(params)
        arr = (Params * self.n)()
        for i, p in enumerate(params):
            arr[i] = p
        self.params = [p.copy() for p in params]
        self.h = C.c_void_p()
        check(self.lib.trapbec_batch_create(self.n, arr, C.byref(self.h)), "trapbec_batch_create")
        fp64 = params[0].precision == abi.FP64
        self.cdtype = np.complex128 if fp64 else np.complex64

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.trapbec_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shape(self, i):
        p = self.params[i]
        return (p.nx, p.ny, p.nz)

    def set_psi(self, i: int, psi: np.ndarray) -> None:
        a = np.ascontiguousarray(psi.reshape(self.shape(i)), dtype=self.cdtype)
        check(self.lib.trapbec_batch_set_psi(self.h, int(i), a.ctypes.data), "trapbec_batch_set_psi")

    def get_psi(self, i: int) -> np.ndarray:
        a = np.empty(self.shape(i), dtype=self.cdtype)
        check(self.lib.trapbec_batch_get_psi(self.h, int(i), a.ctypes.data), "trapbec_batch_get_psi")
        return a

    def init_state(self, i: int, name: str, seed=0, amp=1.0, r_tf2=(0, 0, 0), ring_radius=0.0, core2=0.0,
                   noise_amp=0.0) -> None:
        a = InitArgs()
        a.seed, a.amp, a.ring_radius, a.core2, a.noise_amp = int(seed), float(amp), float(ring_radius), \
            float(core2), float(noise_amp)
        for k in range(3):
            a.r_tf2[k] = float(r_tf2[k])
        check(self.lib.trapbec_batch_init_state(self.h, int(i), name.encode(), C.byref(a)),
              "trapbec_batch_init_state")

    def set_imag_stop(self, mode: int = abi.STOP_REL, energy_scale=None) -> None:
        """abi.STOP_REL: instance i stops at |dE|/|E| <= tol (default).  abi.STOP_ABS: at
        |dE| * energy_scale[i] < tol (energy_scale None: 1 for every instance)."""
        arr = None
        if energy_scale is not None:
            arr = (C.c_double * self.n)(*[float(v) for v in energy_scale])
        check(self.lib.trapbec_batch_set_imag_stop(self.h, int(mode), arr), "trapbec_batch_set_imag_stop")

    def solve(self, max_steps: int, tol: float, check_every: int = 64) -> dict:
        steps = (C.c_int * self.n)()
        e = (C.c_double * self.n)()
        mu = (C.c_double * self.n)()
        check(self.lib.trapbec_batch_solve_imag(self.h, int(max_steps), float(tol), int(check_every), steps, e, mu),
              "trapbec_batch_solve_imag")
        return {"steps": list(steps), "energy": list(e), "mu": list(mu)}

    def status(self, i: int) -> dict:
        o = (C.c_double * 10)()
        check(self.lib.trapbec_batch_status(self.h, int(i), o), "trapbec_batch_status")
        keys = ("scale", "e_prev", "rel", "energy", "mu", "norm", "n0", "step", "converged", "nonfinite")
        return dict(zip(keys, list(o)))

    def stats(self) -> dict:
        ms, tz, ty, nl = C.c_double(0), C.c_int(0), C.c_int(0), C.c_int64(0)
        check(self.lib.trapbec_batch_stats(self.h, C.byref(ms), C.byref(tz), C.byref(ty), C.byref(nl)),
              "trapbec_batch_stats")
        return {"solve_ms": ms.value, "tile_z": tz.value, "tile_y": ty.value, "launches": nl.value}
