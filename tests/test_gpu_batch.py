"""Batched imaginary-time solves against the CPU oracle and the single-grid path."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from trapbec_gb300 import Solver, abi
from trapbec_gb300.batch import BatchSolver
from tests.helpers import params, smooth_state, rel_err

pytestmark = pytest.mark.gpu


def _mixed_params(prec):
    # uneven grids, traps, rotation and steps in one batch
    return [
        params(n=(16, 16, 16), L=(8.0, 8.0, 8.0), prec=prec, pot="harmonic", harm=(64.0, 64.0, 64.0), dt=0.008),
        params(n=(24, 20, 32), L=(12.0, 10.0, 16.0), prec=prec, pot="harmonic", harm=(144.0, 100.0, 64.0),
               dt=0.01, omega=0.25),
        params(n=(12, 16, 64), L=(6.0, 8.0, 32.0), prec=prec, pot="harmonic", harm=(36.0, 64.0, 256.0), dt=0.006),
    ]


def test_batch_matches_oracle_fixed_steps_fp64():
    ps = _mixed_params(abi.FP64)
    b = BatchSolver(ps)
    psis = [smooth_state(p, seed=40 + i) for i, p in enumerate(ps)]
    for i, psi in enumerate(psis):
        b.set_psi(i, psi)
    out = b.solve(max_steps=40, tol=0.0, check_every=8)
    assert out["steps"] == [40, 40, 40]
    for i, p in enumerate(ps):
        o = Oracle(p)
        o.set_psi(psis[i])
        so, _ = o.step_imag_rk3(40, 0.0)
        assert so == 40
        assert rel_err(b.get_psi(i), o.get_psi()) < 1e-11, i


def test_batch_converges_like_single_grid_fp64():
    ps = _mixed_params(abi.FP64)
    b = BatchSolver(ps)
    psis = [smooth_state(p, seed=50 + i) for i, p in enumerate(ps)]
    for i, psi in enumerate(psis):
        b.set_psi(i, psi)
    out = b.solve(max_steps=20000, tol=1e-10, check_every=32)
    for i, p in enumerate(ps):
        s = Solver(p)
        s.set_psi(psis[i])
        steps, rel = s.step_imag(20000, abi.IMAG_RK3_RENORM, 1e-10)
        assert abs(out["steps"][i] - steps) <= 1, (i, out["steps"][i], steps)
        assert steps < 20000
        assert rel_err(b.get_psi(i), s.get_psi()) < 1e-8
        d = s.diag()
        assert abs(out["mu"][i] - d["mu"]) < 1e-8 * abs(d["mu"])


def test_batch_fp32_relaxes_and_counts_launches():
    ps = _mixed_params(abi.FP32)
    b = BatchSolver(ps)
    for i, p in enumerate(ps):
        b.set_psi(i, smooth_state(p, seed=60 + i))
    out = b.solve(max_steps=3000, tol=1e-7, check_every=64)
    st = b.stats()
    assert st["launches"] > 0 and st["tile_z"] in (64, 128)
    for i, p in enumerate(ps):
        o = Oracle(params(n=(p.nx, p.ny, p.nz), L=(p.lx, p.ly, p.lz), pot="harmonic",
                          harm=(p.harm_wx, p.harm_wy, p.harm_wz), dt=p.dt_re, omega=p.omega_z))
        o.set_psi(b.get_psi(i).astype(np.complex128))
        d = o.diag()
        assert abs(out["mu"][i] / d["mu"] - 1) < 1e-5, (i, out["mu"][i], d["mu"])
        assert out["steps"][i] < 3000


def test_batch_stops_at_max_steps_and_one_step_reports_the_start_energy():
    """A solve never runs past max_steps (also when it is not a multiple of
    check_every), and a one-step solve reports the energy of the starting
    state (the stage-1 reduction of the first step)."""
    ps = _mixed_params(abi.FP64)
    psis = [smooth_state(p, seed=60 + i) for i, p in enumerate(ps)]
    b = BatchSolver(ps)
    for i, psi in enumerate(psis):
        b.set_psi(i, psi)
    out = b.solve(max_steps=1, tol=0.0, check_every=200)
    assert out["steps"] == [1, 1, 1]
    for i, p in enumerate(ps):
        s = Solver(p)
        s.set_psi(psis[i])
        e0 = s.diag()["energy"]
        assert abs(out["energy"][i] - e0) < 1e-12 * abs(e0), i
        s.close()
    b2 = BatchSolver(ps)
    for i, psi in enumerate(psis):
        b2.set_psi(i, psi)
    out = b2.solve(max_steps=13, tol=0.0, check_every=4)
    assert out["steps"] == [13, 13, 13]
    for i, p in enumerate(ps):
        o = Oracle(p)
        o.set_psi(psis[i])
        o.step_imag_rk3(13, 0.0)
        assert rel_err(b2.get_psi(i), o.get_psi()) < 1e-11, i


def test_batch_absolute_stop_per_instance_scale_fp64():
    """trapbec_batch_set_imag_stop(ABS): instance i stops when |dE| * scale[i]
    < tol, at the step the single-grid loop with the same scale stops (one
    apart at the threshold); a larger scale means more steps."""
    ps = _mixed_params(abi.FP64)
    psis = [smooth_state(p, seed=70 + i) for i, p in enumerate(ps)]
    scales = [1.0, 10.0, 100.0]   # thresholds |dE| < 1e-8, 1e-9, 1e-10: well above the FP64 noise floor
    tol = 1e-8
    b = BatchSolver(ps)
    for i, psi in enumerate(psis):
        b.set_psi(i, psi)
    b.set_imag_stop(abi.STOP_ABS, scales)
    out = b.solve(max_steps=20000, tol=tol, check_every=32)
    for i, p in enumerate(ps):
        st = b.status(i)
        assert st["converged"] == 1 and st["rel"] < tol
        s = Solver(p)
        s.set_psi(psis[i])
        s.set_imag_stop(abi.STOP_ABS, scales[i])
        steps, rel = s.step_imag(20000, abi.IMAG_RK3_RENORM, tol)
        assert abs(out["steps"][i] - steps) <= 1, (i, out["steps"][i], steps)
        s.close()
    b.set_imag_stop(abi.STOP_REL)
    with pytest.raises(abi.TrapbecError):
        b.set_imag_stop(abi.STOP_ABS, [1.0, 0.0, 1.0])


def test_batch_matches_single_grid_at_workload_sizes():
    """Draws of the batched ground-state workload itself (uneven 64^3 / 96^3 /
    128^3 grids, traps, g and rotation, FP32 state from the TF guess with
    seeded noise): 20 imaginary-time RK3 steps in one batch against each draw
    relaxed alone through the single-grid path."""
    from trapbec_gb300 import units
    draws = units.ground_state_draws(4, 11, grids=(64, 96, 128), precision=abi.FP32)
    assert len({p.n for p, _ in draws}) > 1
    b = BatchSolver([p.to_params() for p, _ in draws])
    for i, (p, ini) in enumerate(draws):
        b.init_state(i, ini["name"], seed=ini["seed"], amp=ini["amp"], r_tf2=ini["r_tf2"],
                     noise_amp=ini["noise_amp"])
    out = b.solve(max_steps=20, tol=0.0, check_every=20)
    assert out["steps"] == [20] * len(draws)
    for i, (p, ini) in enumerate(draws):
        s = Solver(p.to_params())
        s.init_state(ini["name"], seed=ini["seed"], amp=ini["amp"], r_tf2=ini["r_tf2"], noise_amp=ini["noise_amp"])
        steps, _ = s.step_imag(20, abi.IMAG_RK3_RENORM, 0.0)
        assert steps == 20
        a, ref = b.get_psi(i).astype(np.complex128), s.get_psi().astype(np.complex128)
        assert np.linalg.norm(a - ref) / np.linalg.norm(ref) < 1e-6, i
        s.close()
    b.close()
