"""The imaginary-time step bound used to relax the rotating quench's starting
state (reports.imag_step_bound), checked on the oracle (CPU restatement of the
reference's stencil with the RK3 + renormalisation loop): the relaxation stays
stable at the bound and runs away at twice it, so the bound is a safe step
within a factor of two of the real limit."""
import math

import numpy as np

from oracle.pyoracle import Oracle
from trapbec_gb300 import abi, units
from trapbec_gb300.reports import imag_step_bound


def _relaxed_energy(frac, n=24, steps=400):
    prob, _ = units.rotating_quench_512(abi.FP64, n=n)
    p = prob.to_params()
    p.dt_re = 2 * prob.mu * frac * imag_step_bound(prob)
    o = Oracle(p)
    a = abi.InitArgs()
    a.seed, a.amp, a.noise_amp = 5, 1.0, 1e-2
    for k, w in enumerate(prob.omega):
        a.r_tf2[k] = (prob.a * w / math.sqrt(2 * prob.mu)) ** 2
    o.init_state("tf_noise", a)
    o.step_imag_rk3(steps, 0.0)
    return o.diag()["energy"]


def test_imag_step_bound_is_stable_and_within_2x():
    e_safe = _relaxed_energy(0.5)
    e_bound = _relaxed_energy(1.0)
    e_twice = _relaxed_energy(2.0)
    assert np.isfinite(e_bound) and abs(e_bound / e_safe - 1) < 1e-3   # 29641.29 at both
    assert not (np.isfinite(e_twice) and e_twice < 100 * e_safe)       # runs away (~1.3e7)
