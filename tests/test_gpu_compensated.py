"""The compensated FP32 real-time form (TRAPBEC_RK3_COMPENSATED) against the
oracle's compensated RK3 and against the FP64 oracle.

The state is a 32^3 ground state of the rotating-trap workload in the
Thomas-Fermi unit scale, which turns slowly in phase: the plain FP32 update
loses the sub-ulp part of each increment and the norm drifts by 5.5e-6 in 200
steps (the reference's FP32 behaviour, pinned on the oracle in
test_oracle_fp32_gauge.py).  The compensated form keeps those parts in a
remainder array; on the oracle it stays within 1.1e-9 in norm and 3.8e-8 in
L2 of the FP64 run."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from trapbec_gb300 import Solver, abi
from tests.helpers import params, smooth_state
from tests.test_oracle_fp32_gauge import _ground_state

pytestmark = pytest.mark.gpu


def _l2(x, y):
    return float(np.linalg.norm((x - y).ravel()) / np.linalg.norm(y.ravel()))


def _norm(x):
    return float(np.sum(np.abs(x.astype(np.complex128)) ** 2))


@pytest.fixture(scope="module")
def ground():
    prob, psi_ref, _ = _ground_state()
    psi0 = psi_ref.astype(np.complex64)
    o = Oracle(prob.to_params())
    o.set_psi(psi0.astype(np.complex128))
    o.step_rt(200)
    p32 = prob.to_params()
    p32.precision = abi.FP32
    oc = Oracle(p32)
    oc.set_psi(psi0)
    oc.step_rt_comp(200)
    return prob, psi0, o.get_psi(), oc.get_psi().astype(np.complex128)


@pytest.mark.parametrize("shape", [None, (64, 16), (64, 8)])
def test_compensated_form_keeps_the_fp64_norm(ground, shape):
    prob, psi0, ref64, comp_oracle = ground
    p = prob.to_params()
    p.precision = abi.FP32
    s = Solver(p)
    if shape is not None:
        s.set_kernel(2, *shape)
    s.set_stage_form(abi.RK3_COMPENSATED)
    assert s.stage_form() == abi.RK3_COMPENSATED
    s.set_psi(psi0)
    s.step_rt(200)
    got = s.get_psi().astype(np.complex128)
    # tolerances: the oracle's compensated run is 1.1e-9 / 3.8e-8 from FP64
    assert abs(_norm(got) / _norm(ref64) - 1) < 1e-8
    assert _l2(got, ref64) < 1e-7
    assert _l2(got, comp_oracle) < 1e-7
    # the plain FP32 form of the same run drifts (5.5e-6 on the oracle)
    s.set_stage_form(abi.RK3_THREE_STAGE)
    s.set_psi(psi0)
    s.step_rt(200)
    plain = s.get_psi().astype(np.complex128)
    assert _norm(plain) / _norm(ref64) - 1 > 1e-6
    s.close()


def test_compensated_remainder_restarts_with_a_new_state(ground):
    """set_psi starts a new state: its remainders start at zero, so a context
    that ran before gives bit-identical results to a fresh one."""
    prob, psi0, _, _ = ground
    p = prob.to_params()
    p.precision = abi.FP32
    a, b = Solver(p), Solver(p)
    for s in (a, b):
        s.set_stage_form(abi.RK3_COMPENSATED)
    a.set_psi(psi0)
    a.step_rt(30)
    a.set_psi(psi0)
    a.step_rt(40)
    b.set_psi(psi0)
    b.step_rt(25)
    b.step_rt(15)
    assert np.array_equal(a.get_psi(), b.get_psi())
    # the imaginary-time loop changes psi too: the remainders restart after it
    a.step_imag(3, abi.IMAG_RK3_RENORM, 0.0)
    psi1 = a.get_psi()
    a.step_rt(10)
    b.set_psi(psi1)
    b.step_rt(10)
    assert np.array_equal(a.get_psi(), b.get_psi())


def test_compensated_form_where_it_does_not_run():
    p = params(n=(16, 16, 16), L=(8.0, 8.0, 8.0), prec=abi.FP64, pot="harmonic", harm=(6.0, 6.0, 6.0))
    s = Solver(p)
    with pytest.raises(abi.TrapbecError) as e:
        s.set_stage_form(abi.RK3_COMPENSATED)
    assert e.value.code == abi.ERR_UNSUPPORTED
    p32 = params(n=(16, 16, 16), L=(8.0, 8.0, 8.0), prec=abi.FP32, pot="harmonic", harm=(6.0, 6.0, 6.0))
    s32 = Solver(p32)
    s32.set_stage_form(abi.RK3_COMPENSATED)
    s32.set_psi(smooth_state(p32, seed=3).astype(np.complex64))
    s32.set_kernel(1)                       # the per-cell kernel has no compensated stages
    with pytest.raises(abi.TrapbecError) as e:
        s32.step_rt(1)
    assert e.value.code == abi.ERR_UNSUPPORTED
    s32.set_kernel(0)
    s32.step_rt(2)
