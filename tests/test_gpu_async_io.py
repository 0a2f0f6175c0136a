"""Overlapped host copies (trapbec_set_psi_async / trapbec_get_psi_async /
trapbec_step_rt_async): the pipelined call sequence must give the states and
diagnostics of the plain one bit for bit, a queued state must not be seen
before the next time-stepping call, and a timed-out device wait inside
queued steps must still be reported (a wait pointed at an mbarrier phase
nothing completes, as in test_gpu_failures.py; no GPU fault)."""
import ctypes as C

import numpy as np
import pytest

from trapbec_gb300 import Solver, abi
from trapbec_gb300.abi import TrapbecError
from tests.helpers import params, smooth_state

pytestmark = pytest.mark.gpu


def _problem(prec):
    return params(n=(64, 64, 64), L=(16.0, 16.0, 16.0), prec=prec, pot="harmonic", harm=(4.0, 4.0, 4.0),
                  omega=0.3)


def _state(p, seed):
    return smooth_state(p, seed=seed).astype(np.complex64 if p.precision == abi.FP32 else np.complex128)


def _pinned_like(a):
    import torch
    dt = torch.complex64 if a.dtype == np.complex64 else torch.complex128
    t = torch.empty(a.size, dtype=dt, pin_memory=True)
    return t, t.numpy().reshape(a.shape)


@pytest.mark.parametrize("form", [abi.RK3_THREE_STAGE, abi.RK3_PSI_DIFF])
@pytest.mark.parametrize("prec", [abi.FP32, abi.FP64])
def test_pipelined_calls_match_plain_calls(prec, form):
    p = _problem(prec)
    a = _state(p, seed=3)
    b = (a * np.exp(0.3j)).astype(a.dtype)[::-1].copy()
    k = 6
    ref = Solver(p)
    ref.set_stage_form(form)
    ref.set_psi(a)
    ref.step_rt(k)
    want_a, want_da = ref.get_psi(), ref.diag()
    ref.set_psi(b)
    ref.step_rt(k)
    want_b, want_db = ref.get_psi(), ref.diag()

    s = Solver(p)
    s.set_stage_form(form)
    keep_a, host_a = _pinned_like(a)
    keep_b, host_b = _pinned_like(a)
    keep_o1, out_a = _pinned_like(a)
    keep_o2, out_b = _pinned_like(a)
    host_a[...] = a
    host_b[...] = b
    s.set_psi_async(host_a)
    s.step_rt_async(k)
    s.get_psi_async(out_a)
    s.set_psi_async(host_b)          # queued: the diagnostics below still see the stepped first state
    da = s.diag()
    s.step_rt_async(k)
    s.get_psi_async(out_b)
    db = s.diag()
    s.synchronize()
    assert np.array_equal(out_a.view(np.uint8), want_a.view(np.uint8))
    assert np.array_equal(out_b.view(np.uint8), want_b.view(np.uint8))
    assert da == want_da and db == want_db
    assert s.t == ref.t
    assert s.last_kernel_ms() > 0.0
    s.close()

    # two calls deep: the second call's state and steps are queued before the
    # first call's diagnostics and state are read back
    s = Solver(p)
    s.set_stage_form(form)
    out_a[...] = 0
    out_b[...] = 0
    s.set_psi_async(host_a)
    s.step_rt_async(k)
    s.get_psi_async(out_a)
    s.diag_async()
    s.set_psi_async(host_b)
    s.step_rt_async(k)
    da = s.diag_wait()
    s.wait_psi()
    s.get_psi_async(out_b)
    s.diag_async()
    db = s.diag_wait()
    s.synchronize()
    assert np.array_equal(out_a.view(np.uint8), want_a.view(np.uint8))
    assert np.array_equal(out_b.view(np.uint8), want_b.view(np.uint8))
    assert da == want_da and db == want_db
    s.close()
    ref.close()


def test_queued_state_is_replaced_by_set_psi_and_unseen_before_a_step():
    p = _problem(abi.FP32)
    a = _state(p, seed=4)
    b = (a * np.exp(-0.7j)).astype(a.dtype)
    s = Solver(p)
    s.set_psi(a)
    s.set_psi_async(b)
    assert np.array_equal(s.get_psi(), a)        # not applied before a time-stepping call
    s.set_psi(a)                                  # replaces the queued state
    s.step_rt(3)
    ref = Solver(p)
    ref.set_psi(a)
    ref.step_rt(3)
    assert np.array_equal(s.get_psi(), ref.get_psi())
    s.set_psi_async(b)                            # the blocking step takes a queued state too
    s.step_rt(3)
    ref.set_psi(b)
    ref.step_rt(3)
    assert np.array_equal(s.get_psi(), ref.get_psi())
    s.close()
    ref.close()


@pytest.mark.parametrize("n", [(5, 5, 5), (6, 5, 4)])
def test_round_trip_of_odd_sized_states(n):
    """The device copy's 8-byte tail (complex FP32 arrays of odd length) and
    the per-cell kernel path."""
    p = params(n=n, L=(4.0, 4.0, 4.0), prec=abi.FP32, pot="harmonic", harm=(1.0, 1.0, 1.0))
    a = _state(p, seed=5)
    s = Solver(p)
    s.set_psi_async(a)
    s.step_rt_async(0)                            # applies the queued state
    out = np.empty(p.nx * p.ny * p.nz, dtype=np.complex64)
    s.get_psi_async(out)
    s.wait_psi()
    assert np.array_equal(out.reshape(a.shape), a)
    s.step_rt_async(2)
    out2 = np.empty_like(out)
    s.get_psi_async(out2)
    s.synchronize()
    ref = Solver(p)
    ref.set_psi(a)
    ref.step_rt(2)
    assert np.array_equal(out2.reshape(a.shape), ref.get_psi())
    s.close()
    ref.close()


def test_queued_steps_report_a_timed_out_wait():
    p = _problem(abi.FP32)
    a = _state(p, seed=2)
    s = Solver(p)
    s.set_psi(a)
    s.set_wait_limit(1000, inject=True)
    s.step_rt_async(1)                            # queued: the status comes with the next wait
    with pytest.raises(TrapbecError) as e:
        s.synchronize()
    assert e.value.code == abi.ERR_TIMEOUT
    s.step_rt_async(1)                            # the queued diagnostics report it as well
    s.diag_async()
    with pytest.raises(TrapbecError) as e:
        s.diag_wait()
    assert e.value.code == abi.ERR_TIMEOUT
    with pytest.raises(TrapbecError) as e:
        s.synchronize()
    assert e.value.code == abi.ERR_TIMEOUT
    s.set_wait_limit(0, inject=False)
    s.set_psi(a)
    s.step_rt(2)
    assert s.diag()["nonfinite"] == 0
    with pytest.raises(TrapbecError) as e:        # nothing pending
        s.diag_wait()
    assert e.value.code == abi.ERR_STATE
    s.close()


def test_async_calls_take_the_interior_layout_only():
    p = _problem(abi.FP32)
    s = Solver(p)
    buf = np.zeros(tuple(v + 6 for v in s.shape), dtype=np.complex64)
    assert s.lib.trapbec_set_psi_async(s.ctx, buf.ctypes.data, abi.LAYOUT_GHOSTED) == abi.ERR_ARG
    assert s.lib.trapbec_get_psi_async(s.ctx, buf.ctypes.data, abi.LAYOUT_GHOSTED) == abi.ERR_ARG
    assert s.lib.trapbec_set_psi_async(s.ctx, None, abi.LAYOUT_INTERIOR) == abi.ERR_ARG
    assert s.lib.trapbec_wait_psi(s.ctx) == abi.OK
    assert s.lib.trapbec_synchronize(s.ctx) == abi.OK
    assert s.lib.trapbec_synchronize(None) == abi.ERR_ARG
    s.close()


@pytest.mark.parametrize("prec", [abi.FP32, abi.FP64])
def test_host_state_writers_write_the_context_writers_bytes(prec, tmp_path):
    """var####.dat and var.dat from a state read back by get_psi_async
    (trapbec_write_var_host / _restart_host) are the bytes trapbec_write_var /
    trapbec_write_restart write for the same state."""
    import os
    p = _problem(prec)
    s = Solver(p)
    s.set_psi(_state(p, seed=6))
    s.step_rt(2)
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    for d in (a, b):
        os.makedirs(os.path.join(d, "proc000"))
    s.write_var(a, itime=200, shots=100)
    s.write_restart(a, itime=200)
    keep, host = _pinned_like(s.get_psi())
    s.get_psi_async(host)
    s.wait_psi()
    lib = s.lib
    assert lib.trapbec_write_var_host(C.byref(s.params), b.encode(), 200, 100, s.t, 0, host.ctypes.data) == abi.OK
    assert lib.trapbec_write_restart_host(C.byref(s.params), b.encode(), 200, s.t, host.ctypes.data) == abi.OK
    for f in ("var0002.dat", "var.dat"):
        assert open(os.path.join(a, "proc000", f), "rb").read() == open(os.path.join(b, "proc000", f), "rb").read()
    ptr = C.c_void_p()
    assert lib.trapbec_host_alloc(64, C.byref(ptr)) == abi.OK and ptr.value
    lib.trapbec_host_free(ptr)
    assert lib.trapbec_host_alloc(0, C.byref(ptr)) == abi.ERR_ARG
    s.close()
