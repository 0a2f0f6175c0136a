"""Failure detection, exercised without any GPU fault: faults are made on the
host (a NaN seeded into psi, missing / truncated / mismatched restart files,
a wait pointed at an mbarrier phase nothing completes) and the tests check
the status the library returns and that the context stays usable."""
import os
import struct
import subprocess

import numpy as np
import pytest

from trapbec_gb300 import Solver, abi
from trapbec_gb300.abi import TrapbecError
from trapbec_gb300.batch import BatchSolver
from tests.helpers import params, smooth_state

pytestmark = pytest.mark.gpu


def _tiled_problem(prec=abi.FP32):
    return params(n=(64, 64, 64), L=(16.0, 16.0, 16.0), prec=prec, pot="harmonic", harm=(4.0, 4.0, 4.0),
                  omega=0.3)


def test_forced_wait_timeout_returns_status_and_context_recovers():
    p = _tiled_problem()
    psi0 = smooth_state(p, seed=2)
    ref = Solver(p)
    ref.set_psi(psi0)
    ref.step_rt(4)
    want = ref.get_psi()
    s = Solver(p)
    s.set_psi(psi0)
    s.set_wait_limit(1000, inject=True)
    with pytest.raises(TrapbecError) as e:
        s.step_rt(1)
    assert e.value.code == abi.ERR_TIMEOUT
    # the context stays usable: restore the limit and the state, step again
    s.set_wait_limit(0, inject=False)
    s.set_psi(psi0)
    s.t = 0.0
    s.step_rt(4)
    assert np.array_equal(s.get_psi(), want)
    assert s.diag()["nonfinite"] == 0


def test_forced_wait_timeout_in_imaginary_time():
    p = _tiled_problem()
    s = Solver(p)
    s.set_psi(smooth_state(p, seed=3))
    s.set_wait_limit(1000, inject=True)
    with pytest.raises(TrapbecError) as e:
        s.step_imag(3, abi.IMAG_RK3_RENORM, 1e-10)
    assert e.value.code == abi.ERR_TIMEOUT
    s.set_wait_limit(0, inject=False)
    s.set_psi(smooth_state(p, seed=3))
    s.step_imag(3, abi.IMAG_RK3_RENORM, 0.0)
    assert np.isfinite(s.diag()["energy"])


@pytest.mark.parametrize("prec", [abi.FP32, abi.FP64])
def test_nan_seeded_psi_is_reported(prec):
    p = _tiled_problem(prec)
    psi = smooth_state(p, seed=4)
    psi[10, 20, 30] = np.nan
    s = Solver(p)
    s.set_psi(psi)
    assert s.diag()["nonfinite"] == 1
    s.step_rt(2)
    assert s.diag()["nonfinite"] == 1
    s.set_psi(psi)
    with pytest.raises(TrapbecError) as e:
        s.step_imag(5, abi.IMAG_RK3_RENORM, 1e-10)
    assert e.value.code == abi.ERR_NONFINITE
    # a clean state afterwards works
    s.set_psi(smooth_state(p, seed=4))
    s.step_imag(5, abi.IMAG_RK3_RENORM, 0.0)
    assert s.diag()["nonfinite"] == 0


def test_batch_nonfinite_instance_is_reported():
    ps = [params(n=(32, 32, 32), L=(8.0, 8.0, 8.0), pot="harmonic", harm=(4.0, 4.0, 4.0), prec=abi.FP32)
          for _ in range(2)]
    b = BatchSolver(ps)
    good = smooth_state(ps[0], seed=1)
    bad = good.copy()
    bad[3, 4, 5] = np.inf
    b.set_psi(0, good)
    b.set_psi(1, bad)
    with pytest.raises(TrapbecError) as e:
        b.solve(max_steps=20, tol=1e-10)
    assert e.value.code == abi.ERR_NONFINITE
    assert b.status(1)["nonfinite"] > 0


def test_restart_missing_truncated_and_mismatched(tmp_path):
    p = params(n=(16, 16, 16), L=(8.0, 8.0, 8.0), prec=abi.FP32)
    s = Solver(p)
    s.set_psi(smooth_state(p, seed=5))
    with pytest.raises(TrapbecError) as e:
        s.read_restart(str(tmp_path / "empty"))
    assert e.value.code == abi.ERR_IO
    d = tmp_path / "data"
    s.write_restart(str(d), 100)
    f = d / "proc000" / "var.dat"
    raw = f.read_bytes()
    f.write_bytes(raw[:len(raw) // 2])                     # truncated
    with pytest.raises(TrapbecError) as e:
        s.read_restart(str(d))
    assert e.value.code == abi.ERR_IO
    q = params(n=(16, 16, 8), L=(8.0, 8.0, 8.0), prec=abi.FP32)   # another grid's file
    s2 = Solver(q)
    s2.set_psi(smooth_state(q, seed=5))
    s2.write_restart(str(d), 100)
    with pytest.raises(TrapbecError) as e:
        s.read_restart(str(d))
    assert e.value.code == abi.ERR_IO
    s.write_restart(str(d), 100)                           # and a good one reads back
    assert s.read_restart(str(d)) == 101


def test_driver_stops_with_error_file_on_nonfinite_restart(tmp_path):
    from tests.test_driver import CPARAM, _run
    from trapbec_gb300 import parse_cparam
    p = parse_cparam(CPARAM.format(nsteps=20))
    p.precision = abi.FP32
    s = Solver(p)
    psi = smooth_state(p, seed=6)
    psi[1, 2, 3] = np.nan
    s.set_psi(psi)
    s.write_restart(str(tmp_path / "data"), 5)
    r = _run(tmp_path, CPARAM.format(nsteps=20))
    assert r.returncode == 1
    assert "non-finite" in (tmp_path / "ERROR").read_text()


def test_bad_arguments_return_status_and_leave_the_context_usable():
    """Invalid arguments to the kernel-selection and form entry points are
    error codes (never a launch), and the context keeps stepping afterwards."""
    import ctypes as C
    from trapbec_gb300 import Solver
    p = params(n=(12, 32, 128), L=(6.0, 16.0, 64.0), prec=abi.FP32, pot="harmonic", harm=(3.0, 4.0, 5.0),
               omega=0.2, dt=0.01)
    s = Solver(p)
    lib = s.lib
    assert lib.trapbec_set_kernel(s.ctx, 3, 0, 0) == abi.ERR_ARG            # no such kernel kind
    assert lib.trapbec_set_kernel(s.ctx, 2, -99, 0) == abi.ERR_UNSUPPORTED  # no such built shape
    assert lib.trapbec_set_kernel(s.ctx, 2, 48, 48) == abi.ERR_UNSUPPORTED  # no shape of this size
    assert lib.trapbec_set_stage_form(s.ctx, 4) == abi.ERR_ARG   # no such form
    assert lib.trapbec_set_chunk(s.ctx, -2 ** 31) == abi.ERR_ARG   # negative: the strided order; INT_MIN: none
    tz, ty = C.c_int(0), C.c_int(0)
    assert lib.trapbec_get_tile_shape(s.ctx, 1, None, C.byref(ty)) == abi.ERR_ARG
    assert lib.trapbec_get_tile_shape(s.ctx, 1, C.byref(tz), C.byref(ty)) == abi.OK
    assert (tz.value, ty.value) == (64, 32)
    s.set_psi(smooth_state(p, seed=3))
    n0 = s.diag()["intpsi2"]
    s.step_rt(5)
    assert abs(s.diag()["intpsi2"] / n0 - 1) < 1e-4
