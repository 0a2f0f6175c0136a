"""ctypes mirror of include/trapbec.h and the loader of libtrapbec.so.

The library is the product: there is no Python or CPU fallback.  If the
shared object is missing, `load()` raises; build it with
`trapbec_gb300.build.build_library()` (or `__graft_entry__.build()`).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libtrapbec.so")

# ---- enumerations (trapbec.h) ---------------------------------------------
OK = 0
ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_TIMEOUT = 1, 2, 3, 4, 5
ERR_NONFINITE, ERR_IO, ERR_UNSUPPORTED, ERR_PARSE, ERR_NODEVICE = 6, 7, 8, 9, 10

BC_ZERO, BC_SOLID, BC_PERIODIC = 0, 1, 2
BOUNDARIES = {"zero": BC_ZERO, "solid": BC_SOLID, "periodic": BC_PERIODIC}

POTENTIALS = {
    "zero": 0, "harmonic": 1, "harmonic_ring": 2, "harmonic_ring2": 3,
    "barrier": 4, "box_trap": 5, "channel": 6, "quartic": 7, "sphere": 8,
    "mobius": 9, "array": 10,
}
POT_ZERO, POT_HARMONIC, POT_MOBIUS, POT_ARRAY = 0, 1, 9, 10

FP32, FP64 = 0, 1
LAYOUT_INTERIOR, LAYOUT_GHOSTED = 0, 1
FIELD_VELOCITY, FIELD_QPRESSURE = 0, 1
IMAG_REF_EULER, IMAG_RK3_RENORM = 0, 1
STOP_REL, STOP_ABS, STOP_ABS_PER_NORM = 0, 1, 2
RK3_THREE_STAGE, RK3_DEFERRED, RK3_COMPENSATED, RK3_PSI_DIFF = 0, 1, 2, 3

SCALAR_OMEGA_Z, SCALAR_DT_RE, SCALAR_DT_IM, SCALAR_GAMMA = 0, 1, 2, 3
SCALAR_T, SCALAR_ADVECTIVE_VX, SCALAR_NORM_TARGET = 4, 5, 6


class Params(C.Structure):
    """struct trapbec_params (trapbec.h); names follow cparam.local."""

    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("nprocx", C.c_int32), ("nprocy", C.c_int32),
        ("precision", C.c_int32), ("boundaries", C.c_int32),
        ("periodicz", C.c_int32), ("two_dim", C.c_int32),
        ("potential", C.c_int32), ("lbeam", C.c_int32),
        ("winding_number", C.c_int32),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("dt_re", C.c_double), ("dt_im", C.c_double), ("gamma", C.c_double),
        ("harm_wx", C.c_double), ("harm_wy", C.c_double), ("harm_wz", C.c_double),
        ("potential_off", C.c_double), ("wbeam", C.c_double),
        ("advective_vx", C.c_double), ("omega_z", C.c_double),
        ("t_spindown", C.c_double), ("ring_rad", C.c_double),
        ("vor_ring_count", C.c_int32), ("reserved", C.c_int32 * 7),
    ]

    def copy(self) -> "Params":
        q = Params()
        C.pointer(q)[0] = self
        return q

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class DiagOut(C.Structure):
    """struct trapbec_diag_out."""

    _fields_ = [
        ("intpsi2", C.c_double), ("maxpsi", C.c_double), ("minpsi", C.c_double),
        ("meanpsi", C.c_double), ("norm", C.c_double), ("energy", C.c_double),
        ("mu", C.c_double), ("kinetic", C.c_double), ("potential", C.c_double),
        ("interaction", C.c_double), ("rotation", C.c_double),
        ("nonfinite", C.c_int32), ("reserved", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class InitArgs(C.Structure):
    """struct trapbec_init_args."""

    _fields_ = [
        ("seed", C.c_uint64), ("amp", C.c_double), ("r_tf2", C.c_double * 3),
        ("ring_radius", C.c_double), ("core2", C.c_double),
        ("noise_amp", C.c_double), ("reserved", C.c_double * 4),
    ]


def default_params() -> Params:
    """Defaults mirroring trapbec_params_default() (checked against it in tests)."""
    p = Params()
    p.nx = p.ny = p.nz = 64
    p.nprocx = p.nprocy = 1
    p.precision = FP64
    p.boundaries = BC_ZERO
    p.periodicz = 0
    p.two_dim = 0
    p.potential = POT_HARMONIC
    p.lbeam = 0
    p.winding_number = 1
    p.lx = p.ly = p.lz = 32.0
    p.dt_re, p.dt_im = 0.005, 0.0
    p.gamma = 0.0
    p.harm_wx = p.harm_wy = p.harm_wz = 0.0
    p.potential_off = 3.4028234663852886e38  # huge(1.) of a default real
    p.wbeam = 4.0
    p.advective_vx = 0.0
    p.omega_z = 0.0
    p.t_spindown = 3.4028234663852886e38
    p.ring_rad = 10.0
    p.vor_ring_count = 1
    return p


# ---- function prototypes ---------------------------------------------------
_VP = C.c_void_p
_PROTOS = {
    "trapbec_params_default": (C.c_int, [C.POINTER(Params)]),
    "trapbec_params_parse": (C.c_int, [C.c_char_p, C.POINTER(Params), C.c_char_p, C.c_size_t]),
    "trapbec_create": (C.c_int, [C.POINTER(Params), C.POINTER(_VP)]),
    "trapbec_destroy": (None, [_VP]),
    "trapbec_set_psi": (C.c_int, [_VP, _VP, C.c_int]),
    "trapbec_get_psi": (C.c_int, [_VP, _VP, C.c_int]),
    "trapbec_set_trap": (C.c_int, [_VP, C.POINTER(C.c_double)]),
    "trapbec_init_state": (C.c_int, [_VP, C.c_char_p, C.POINTER(InitArgs)]),
    "trapbec_get_rhs": (C.c_int, [_VP, _VP]),
    "trapbec_step_rt": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_double)]),
    "trapbec_set_psi_async": (C.c_int, [_VP, _VP, C.c_int]),
    "trapbec_get_psi_async": (C.c_int, [_VP, _VP, C.c_int]),
    "trapbec_step_rt_async": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_double)]),
    "trapbec_wait_psi": (C.c_int, [_VP]),
    "trapbec_synchronize": (C.c_int, [_VP]),
    "trapbec_step_imag": (C.c_int, [_VP, C.c_int, C.c_int, C.c_double,
                                    C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "trapbec_set_imag_stop": (C.c_int, [_VP, C.c_int, C.c_double]),
    "trapbec_diag": (C.c_int, [_VP, C.POINTER(DiagOut)]),
    "trapbec_diag_async": (C.c_int, [_VP]),
    "trapbec_diag_wait": (C.c_int, [_VP, C.POINTER(DiagOut)]),
    "trapbec_set_wait_limit": (C.c_int, [_VP, C.c_uint32, C.c_int]),
    "trapbec_force_vortex": (C.c_int, [_VP, C.c_double, C.c_double, C.c_double]),
    "trapbec_force_random_points": (C.c_int, [_VP, C.c_uint64, C.c_uint64, C.POINTER(C.c_double)]),
    "trapbec_get_velocity": (C.c_int, [_VP, _VP]),
    "trapbec_get_qpressure": (C.c_int, [_VP, _VP]),
    "trapbec_set_scalar": (C.c_int, [_VP, C.c_int, C.c_double]),
    "trapbec_get_scalar": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_double)]),
    "trapbec_set_kernel": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int]),
    "trapbec_set_chunk": (C.c_int, [_VP, C.c_int]),
    "trapbec_set_stage_form": (C.c_int, [_VP, C.c_int]),
    "trapbec_get_tile_shape": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "trapbec_get_stage_form": (C.c_int, [_VP, C.POINTER(C.c_int)]),
    "trapbec_autotune": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_double)]),
    "trapbec_launch_count": (C.c_int, [_VP, C.POINTER(C.c_int64)]),
    "trapbec_last_kernel_ms": (C.c_int, [_VP, C.POINTER(C.c_double)]),
    "trapbec_write_var": (C.c_int, [_VP, C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_int]),
    "trapbec_write_restart": (C.c_int, [_VP, C.c_char_p, C.c_int, C.c_double]),
    "trapbec_write_var_host": (C.c_int, [C.POINTER(Params), C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_int,
                                         _VP]),
    "trapbec_write_restart_host": (C.c_int, [C.POINTER(Params), C.c_char_p, C.c_int, C.c_double, _VP]),
    "trapbec_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(_VP)]),
    "trapbec_host_free": (None, [_VP]),
    "trapbec_write_field": (C.c_int, [_VP, C.c_char_p, C.c_int, C.c_int, C.c_int]),
    "trapbec_read_restart": (C.c_int, [_VP, C.c_char_p, C.POINTER(C.c_int),
                                       C.POINTER(C.c_double)]),
    "trapbec_write_dims": (C.c_int, [C.POINTER(Params), C.c_char_p]),
    "trapbec_write_timing": (C.c_int, [C.POINTER(Params), C.c_char_p, C.c_double, C.c_double]),
    "trapbec_psi_stats_noalloc": (C.c_int, [_VP, C.c_int64, C.c_int, _VP, _VP]),
    "trapbec_batch_create": (C.c_int, [C.c_int, C.POINTER(Params), C.POINTER(_VP)]),
    "trapbec_batch_destroy": (None, [_VP]),
    "trapbec_batch_set_psi": (C.c_int, [_VP, C.c_int, _VP]),
    "trapbec_batch_get_psi": (C.c_int, [_VP, C.c_int, _VP]),
    "trapbec_batch_solve_imag": (C.c_int, [_VP, C.c_int, C.c_double, C.c_int,
                                           C.POINTER(C.c_int), C.POINTER(C.c_double),
                                           C.POINTER(C.c_double)]),
    "trapbec_batch_set_imag_stop": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_double)]),
    "trapbec_batch_init_state": (C.c_int, [_VP, C.c_int, C.c_char_p, C.POINTER(InitArgs)]),
    "trapbec_batch_stats": (C.c_int, [_VP, C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_int64)]),
    "trapbec_batch_status": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_double)]),
    "trapbec_fp64_fma_rate": (C.c_int, [C.POINTER(C.c_double)]),
    "trapbec_strerror": (C.c_char_p, [C.c_int]),
    "trapbec_last_error": (C.c_char_p, []),
    "trapbec_abi_version": (C.c_int, []),
    "trapbec_abi_struct_size": (C.c_int, [C.c_int]),
    # learned warm start (include/trapbec_surrogate.h)
    "tbsg_conv3_fwd": (C.c_int, [_VP, C.c_int, _VP, _VP, _VP, _VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int,
                                 C.c_int, C.c_int, C.c_int, C.c_float, _VP]),
    "tbsg_conv3_dgrad_act": (C.c_int, [_VP, C.c_int, _VP, _VP, _VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_float, _VP]),
    "tbsg_set_conv_path": (C.c_int, [C.c_int]),
    "tbsg_tc_status": (C.c_int, [C.POINTER(C.c_int)]),
    "tbsg_conv3_wgrad_scratch_bytes": (C.c_size_t, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "tbsg_conv3_wgrad": (C.c_int, [_VP, C.c_int, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _VP, _VP, _VP,
                                   C.c_size_t, _VP]),
    "tbsg_weight_prep": (C.c_int, [_VP, _VP, _VP, C.c_int, C.c_int, _VP]),
    "tbsg_act_bwd": (C.c_int, [_VP, _VP, _VP, _VP, C.c_size_t, C.c_float, _VP]),
    "tbsg_pool2_fwd": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _VP]),
    "tbsg_pool2_bwd": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _VP]),
    "tbsg_up2_fwd": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _VP]),
    "tbsg_up2_bwd": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _VP]),
    "tbsg_head_fwd": (C.c_int, [_VP, C.c_int, _VP, _VP, _VP, _VP, C.c_size_t, _VP]),
    "tbsg_head_partials": (C.c_size_t, [C.c_size_t, C.c_int]),
    "tbsg_head_loss": (C.c_int, [_VP, C.c_int, _VP, _VP, _VP, _VP, C.c_size_t, _VP, _VP, _VP, _VP]),
    "tbsg_head_loss_act": (C.c_int, [_VP, _VP, _VP, _VP, _VP, C.c_size_t, _VP, C.c_float, _VP, _VP, _VP]),
    "tbsg_pool2_bwd_act": (C.c_int, [_VP, _VP, _VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                     _VP]),
    "tbsg_up2_bwd_act": (C.c_int, [_VP, _VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, _VP]),
    "tbsg_adam": (C.c_int, [_VP, _VP, _VP, _VP, C.c_size_t, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                            C.c_int, _VP, _VP]),
    "tbsg_clip_scale": (C.c_int, [_VP, C.c_size_t, C.c_float, _VP, _VP, _VP]),
    "tbsg_f32_to_bf16": (C.c_int, [_VP, _VP, C.c_size_t, _VP]),
    "tbsg_features": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                C.c_double, C.c_double, C.c_double, _VP, _VP]),
}

_lib = None
_lock = threading.Lock()


def exported_names() -> list[str]:
    return sorted(_PROTOS)


def load(path: str | None = None) -> C.CDLL:
    """Load libtrapbec.so and attach prototypes.  Raises if it is missing."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                f"libtrapbec.so not found at {p}: build it first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = C.CDLL(p)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


class TrapbecError(RuntimeError):
    def __init__(self, code: int, where: str):
        lib = load()
        msg = lib.trapbec_strerror(code).decode()
        detail = (lib.trapbec_last_error() or b"").decode()
        super().__init__(f"{where}: {msg} ({code}): {detail}")
        self.code = code


def check(code: int, where: str) -> None:
    if code != OK:
        raise TrapbecError(code, where)
