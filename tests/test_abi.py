"""C ABI checks that need no GPU: the library loads, exports every function
include/trapbec.h and include/trapbec_surrogate.h declare, its structs match the Python mirrors, and the
host-only entry points (defaults, cparam.local parser, dims/timing writers)
behave like the reference."""
import ctypes as C
import os
import re

import pytest

from trapbec_gb300 import abi
from trapbec_gb300.abi import Params, DiagOut, InitArgs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("trapbec.h", "trapbec_surrogate.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b((?:trapbec|tbsg)_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_exports_every_declared_symbol():
    lib = C.CDLL(abi.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(abi.exported_names())


def test_struct_sizes_match():
    lib = abi.load()
    assert lib.trapbec_abi_struct_size(0) == C.sizeof(Params)
    assert lib.trapbec_abi_struct_size(1) == C.sizeof(DiagOut)
    assert lib.trapbec_abi_struct_size(2) == C.sizeof(InitArgs)
    assert lib.trapbec_abi_version() == 1


def test_defaults_match_python_mirror():
    lib = abi.load()
    p = Params()
    assert lib.trapbec_params_default(C.byref(p)) == 0
    assert p.as_dict() == abi.default_params().as_dict()


SAMPLE = """!/* sample in the syntax of cparam.local */
real  :: Lx=40., Ly=40., Lz=20
integer, parameter :: Nx=128, Ny=128, Nz=64
complex :: dt=0.01
integer, parameter :: shots=50
character(len=*), parameter :: boundaries='solid'
logical, parameter :: periodicz=.false.
character(len=*), parameter :: init_cond='single_vortex'
character(len=*), parameter :: potential='harmonic'
real, parameter :: harm_wx=12, harm_wy=13., harm_wz=1.5d1 !trap
real, parameter :: potential_off=huge(1.)
real, parameter :: gamma=0.003 !dissipation
logical, parameter :: two_dim=.false.
real, parameter :: omega_z=0.25
"""


def test_cparam_parser():
    from trapbec_gb300 import parse_cparam
    p = parse_cparam(SAMPLE)
    assert (p.nx, p.ny, p.nz) == (128, 128, 64)
    assert (p.lx, p.ly, p.lz) == (40.0, 40.0, 20.0)
    assert p.dt_re == 0.01 and p.dt_im == 0.0
    assert p.boundaries == abi.BC_SOLID and p.periodicz == 0
    assert p.potential == abi.POT_HARMONIC
    assert (p.harm_wx, p.harm_wy, p.harm_wz) == (12.0, 13.0, 15.0)
    assert p.gamma == 0.003 and p.omega_z == 0.25
    assert p.potential_off > 1e38
    q = parse_cparam("complex :: dt=(0.02,-0.001)")
    assert (q.dt_re, q.dt_im) == (0.02, -0.001)


@pytest.mark.parametrize("text,frag", [
    ("character(len=*), parameter :: boundaries='sticky'", "wrong boundaries"),
    ("character(len=*), parameter :: potential='donut'", "incorrect potential"),
    ("real :: bogus_name=1.0", "unknown parameter"),
    ("real :: Lx", "no value"),
    ("logical :: two_dim=yes", "bad value"),
])
def test_cparam_parser_errors(text, frag):
    lib = abi.load()
    p = abi.default_params()
    err = C.create_string_buffer(256)
    rc = lib.trapbec_params_parse(text.encode(), C.byref(p), err, 256)
    assert rc == abi.ERR_PARSE
    assert frag in err.value.decode()


def test_dims_and_timing_logs(tmp_path):
    lib = abi.load()
    p = abi.default_params()
    p.nx, p.ny, p.nz, p.nprocx, p.nprocy = 64, 32, 16, 2, 2
    assert lib.trapbec_write_dims(C.byref(p), str(tmp_path).encode()) == 0
    vals = [int(v) for v in open(tmp_path / "dims.log").read().split()]
    assert vals == [64, 32, 16, 2, 2, 32, 16, 16]   # output.f90:48-60
    assert lib.trapbec_write_timing(C.byref(p), str(tmp_path).encode(), 1.5e-3, 0.25) == 0
    lines = open(tmp_path / "timing.log").read().splitlines()
    f = lines[0].split()
    assert int(f[0]) == 64 * 32 * 16 and int(f[1]) == 4 and abs(float(f[2]) - 1.5e-3) < 1e-12
    assert "communication timing" in lines[1]


def test_create_validates_before_touching_the_device():
    lib = abi.load()
    p = abi.default_params()
    p.nx = 0
    ctx = C.c_void_p()
    assert lib.trapbec_create(C.byref(p), C.byref(ctx)) == abi.ERR_ARG
    p = abi.default_params()
    p.nx, p.nprocx = 30, 4  # uneven split, mpi_var.f90:157-160
    assert lib.trapbec_create(C.byref(p), C.byref(ctx)) == abi.ERR_ARG
    assert b"evenly" in lib.trapbec_last_error()


def test_no_device_fails_loudly(has_gpu):
    if has_gpu:
        pytest.skip("a GPU is present")
    lib = abi.load()
    p = abi.default_params()
    ctx = C.c_void_p()
    rc = lib.trapbec_create(C.byref(p), C.byref(ctx))
    assert rc in (abi.ERR_NODEVICE, abi.ERR_CUDA)
    assert not ctx.value


def test_noalloc_rejects_bad_arguments_before_touching_the_gpu():
    """trapbec_psi_stats_noalloc validates its pointers, precision and size on
    the host and returns TRAPBEC_ERR_ARG without any CUDA call, so this runs
    with no GPU: null, misaligned (psi must hold whole complex values, stats
    doubles), oversized and empty inputs, and an unknown precision."""
    lib = abi.load()
    ok = C.c_void_p(256)          # aligned for both precisions; never dereferenced here
    f = lib.trapbec_psi_stats_noalloc
    assert f(ok, 1 << 29, abi.FP32, ok, None) == abi.ERR_ARG
    assert b"ncells" in lib.trapbec_last_error()
    assert f(ok, 0, abi.FP32, ok, None) == abi.ERR_ARG
    assert f(None, 10, abi.FP32, ok, None) == abi.ERR_ARG
    assert f(ok, 10, abi.FP32, None, None) == abi.ERR_ARG
    assert f(ok, 10, 7, ok, None) == abi.ERR_ARG
    assert f(C.c_void_p(260), 10, abi.FP32, ok, None) == abi.ERR_ARG      # 4-byte aligned psi
    assert b"aligned" in lib.trapbec_last_error()
    assert f(C.c_void_p(264), 10, abi.FP64, ok, None) == abi.ERR_ARG      # 8-byte aligned FP64 psi
    assert b"16 bytes" in lib.trapbec_last_error()
    assert f(ok, 10, abi.FP32, C.c_void_p(260), None) == abi.ERR_ARG      # 4-byte aligned stats
    assert b"stats" in lib.trapbec_last_error()
