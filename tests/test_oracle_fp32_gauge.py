"""FP32 time stepping of a stationary state, in the reference's own
arithmetic (the CPU restatement, no GPU).

A ground state turns its phase by dt' (mu_state - 1/2) per step in the
reference units, whose equation has the chemical potential 1/2 folded in
(i dpsi/dt' = -1/2 lap psi + 1/2 (pot + |psi|^2 - 1) psi).  Under that slow
rotation the real part of psi should fall by half the square of the phase
turned, which in FP32 is below half an ulp in most cells: round-to-nearest
keeps the old value and the norm grows with the square of the phase turned.
Choosing the unit scale at the state's own chemical potential makes the
state stationary in the units the kernels run in, and the bias goes away.
These checks pin that behaviour on the oracle, so the same numbers from the
GPU's FP32 path read as the algorithm's, not the kernel's."""
import math

import numpy as np

from oracle.pyoracle import Oracle
from trapbec_gb300 import abi, units
from trapbec_gb300.reports import imag_step_bound


def _ground_state(n=32, L=128.0):
    prob, _ = units.rotating_quench_512(abi.FP64, n=n)
    prob.box = (L, L, L)
    pr = prob.to_params()
    pr.dt_re = 2 * prob.mu * 0.7 * imag_step_bound(prob)
    o = Oracle(pr)
    a = abi.InitArgs()
    a.seed, a.amp, a.noise_amp = 5, 1.0, 1e-2
    for k, w in enumerate(prob.omega):
        a.r_tf2[k] = (prob.a * w / math.sqrt(2 * prob.mu)) ** 2
    o.init_state("tf_noise", a)
    steps, rel = o.step_imag_rk3(300, 1e-12)
    assert rel < 1e-9
    return prob, o.get_psi(), o.diag()["mu"]


def _drift(prob, psi0, mu_unit, prec, steps=200):
    start = (psi0 * math.sqrt(prob.mu / mu_unit)).astype(np.complex64)
    pg = units.TrapProblem(n=prob.n, box=prob.box, omega=prob.omega, g=prob.g, mu=mu_unit, dt=prob.dt,
                           precision=prec)
    o = Oracle(pg.to_params())
    o.set_psi(start.astype(np.complex128) if prec == abi.FP64 else start)
    n0 = o.diag()["norm"]
    o.step_rt(steps)
    return o.diag()["norm"] / n0 - 1.0


def test_fp32_norm_bias_follows_the_unit_scale():
    prob, psi0, mu_ref = _ground_state()
    assert abs(mu_ref - 0.5) > 1e-3           # the Thomas-Fermi unit scale is off the state's mu
    mu_state = prob.mu_to_trap(mu_ref)
    for mu_unit in (prob.mu, mu_state):
        assert abs(_drift(prob, psi0, mu_unit, abi.FP64)) < 1e-12
    tf32 = _drift(prob, psi0, prob.mu, abi.FP32)
    st32 = _drift(prob, psi0, mu_state, abi.FP32)
    assert tf32 > 1e-6                         # 5.5e-6 after 200 steps
    assert abs(st32) < 1e-7                    # 1.7e-8
