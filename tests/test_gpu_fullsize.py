"""Size-independent properties of the real-time RK3 at the workload's full
size: the 512^3 rotating-trap quench in complex FP32, 1 GiB per array, where
the oracle would take minutes per step.  From the workload's start state (the
seeded Thomas-Fermi cloud with 1e-2 phase noise) in a rotating frame:
- the psi-difference form and the three-stage form, two different sets of
  stage kernels for the same scheme, agree to FP32 rounding;
- the evolution commutes with a global phase (the equation is U(1)-invariant);
- the evolution commutes with the rotation by pi about the trap axis,
  (x, y) -> (-x, -y), which maps the cell-centred grid, the harmonic trap,
  the rotating-frame term x d/dy - y d/dx and the zero boundaries onto
  themselves;
- and, over 2 steps (the oracle's C++ restatement on all host cores, about a
  second per step at this size), both forms match the oracle itself; so does
  the headline form at the 1024^3 stretch size, and the FP64 path at the
  vortex-ring workload's 256^3 to 1e-12.
Tolerances are relative L2 norms of the difference (FP32 rounding over the
steps taken), and 1e-6 on the FP64 norm and energy of the diagnostics.
Measured on a GB300: forms 2.2e-7, phase 1.9e-7, rotation 6.1e-8 (the grid's
FP32 cell-centre coordinates are not exactly odd), against a relative change
of the state of 5.6e-2 over the 20 steps."""
import numpy as np
import pytest

from trapbec_gb300 import Solver, abi, units

pytestmark = pytest.mark.gpu

STEPS = 20
L2_TOL = 2e-6
DIAG_TOL = 1e-6


def _solver(form):
    prob, init = units.rotating_quench_512(abi.FP32)
    p = prob.to_params()
    p.omega_z = prob.omega_z_for(0.5 * init["omega_final"])   # mid-ramp rotation
    s = Solver(p)
    s.set_stage_form(form)
    return s, init


@pytest.fixture(scope="module")
def start():
    s, init = _solver(abi.RK3_PSI_DIFF)
    s.init_state(init["name"], seed=init["seed"], amp=init["amp"], r_tf2=init["r_tf2"],
                 noise_amp=init["noise_amp"])
    psi = s.get_psi()
    s.close()
    return psi


def _run(psi, form, steps=STEPS):
    s, _ = _solver(form)
    s.set_psi(psi)
    s.step_rt(steps)
    out, d = s.get_psi(), s.diag()
    s.close()
    return out, d


def _l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _same_diag(d, ref):
    for k in ("norm", "energy"):
        assert abs(d[k] - ref[k]) <= DIAG_TOL * abs(ref[k]), (k, d[k], ref[k])


@pytest.fixture(scope="module")
def reference_run(start):
    return _run(start, abi.RK3_PSI_DIFF)


def test_forms_agree_at_full_size(start, reference_run):
    a, da = reference_run
    b, db = _run(start, abi.RK3_THREE_STAGE)
    assert a.shape == (512, 512, 512)
    assert _l2(a, b) < L2_TOL
    _same_diag(da, db)


def test_global_phase_commutes_with_the_step(start, reference_run):
    a, da = reference_run
    ph = np.complex64(np.exp(0.7j))
    b, db = _run(start * ph, abi.RK3_PSI_DIFF)
    assert _l2(b, a * ph) < L2_TOL
    _same_diag(db, da)


def test_rotation_by_pi_about_the_trap_axis_commutes_with_the_step(start, reference_run):
    a, da = reference_run
    b, db = _run(np.ascontiguousarray(start[::-1, ::-1, :]), abi.RK3_PSI_DIFF)
    assert _l2(np.ascontiguousarray(b[::-1, ::-1, :]), a) < L2_TOL
    _same_diag(db, da)


def test_both_forms_match_the_oracle_at_full_size(start):
    from oracle.pyoracle import Oracle
    Oracle.set_threads(Oracle.max_threads())
    s, _ = _solver(abi.RK3_PSI_DIFF)
    o = Oracle(s.params)
    s.close()
    o.set_psi(start)
    o.step_rt(2)
    want, dw = o.get_psi(), o.diag()
    for form in (abi.RK3_PSI_DIFF, abi.RK3_THREE_STAGE):
        got, dg = _run(start, form, steps=2)
        assert _l2(got, want) < L2_TOL, form
        _same_diag(dg, dw)


def test_psi_diff_matches_the_oracle_at_the_1024_stretch_size():
    """The workload's largest size, 1024^3 (8 GiB per complex FP32 array, so
    byte offsets into a state run past 2^32): 2 steps of the headline form
    against the oracle from the seeded start state."""
    from oracle.pyoracle import Oracle
    Oracle.set_threads(Oracle.max_threads())
    prob, init = units.rotating_quench_512(abi.FP32, n=1024)
    p = prob.to_params()
    p.omega_z = prob.omega_z_for(0.5 * init["omega_final"])
    s = Solver(p)
    s.set_stage_form(abi.RK3_PSI_DIFF)
    s.init_state(init["name"], seed=init["seed"], amp=init["amp"], r_tf2=init["r_tf2"],
                 noise_amp=init["noise_amp"])
    psi = s.get_psi()
    s.step_rt(2)
    got, dg = s.get_psi(), s.diag()
    s.close()
    assert got.shape == (1024, 1024, 1024)
    o = Oracle(p)
    o.set_psi(psi)
    del psi
    o.step_rt(2)
    want, dw = o.get_psi(), o.diag()
    del o
    assert _l2(got, want) < L2_TOL
    _same_diag(dg, dw)


def test_fp64_matches_the_oracle_to_1e12_at_the_256_ring_size():
    """The FP64 path at the vortex-ring workload's full size (256^3 on
    [-32,32]^3, anisotropic trap, TF background times a ring of radius 8 with
    1e-3 phase noise): 10 steps against the FP64 oracle, 1e-12 relative in
    psi (max norm), norm and energy."""
    from oracle.pyoracle import Oracle
    Oracle.set_threads(Oracle.max_threads())
    prob, init = units.vortex_ring_256(abi.FP64)
    p = prob.to_params()
    s = Solver(p)
    s.init_state(init["name"], seed=init["seed"], amp=init["amp"], r_tf2=init["r_tf2"],
                 ring_radius=init["ring_radius"], noise_amp=init["noise_amp"])
    psi = s.get_psi()
    s.step_rt(10)
    got, dg = s.get_psi(), s.diag()
    s.close()
    o = Oracle(p)
    o.set_psi(psi)
    o.step_rt(10)
    want, dw = o.get_psi(), o.diag()
    assert float(np.max(np.abs(got - want)) / np.max(np.abs(want))) < 1e-12
    for k in ("norm", "energy"):
        assert abs(dg[k] - dw[k]) <= 1e-12 * abs(dw[k]), (k, dg[k], dw[k])
