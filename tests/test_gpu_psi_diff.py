"""The psi-difference real-time RK3 form (TRAPBEC_RK3_PSI_DIFF) against the
CPU oracle's three-stage RK3 (run.f90:42-57).

The form stores no w array: the two psi arrays hold the last two stage
values and each stage recovers the w of the stage before it as
(psi_k - psi_{k-1}) / B_prev.  In exact arithmetic that is the same scheme;
in floating point the recovered w carries the rounding of the psi update it
came from, so FP64 results agree with the reference to a few ulps per step
(the 1e-12 tolerance of the FP64 parity tests), not bit for bit."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from trapbec_gb300 import Solver, abi, units
from tests.helpers import params, smooth_state, rel_err
from tests.test_gpu_tiled import SHAPES, _grid_for

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12

CASES = [(prec, shp, bc, zper) for prec in (abi.FP64, abi.FP32) for shp in SHAPES[prec]
         for bc, zper in ((abi.BC_ZERO, 0), (abi.BC_SOLID, 0), (abi.BC_PERIODIC, 0), (abi.BC_ZERO, 1))]


@pytest.mark.parametrize("prec,shape,bc,zper", CASES, ids=lambda v: str(v))
def test_psi_diff_matches_oracle(prec, shape, bc, zper):
    """Every tile shape and boundary type (ghost fix-ups of boundary tiles
    included), rotating frame and harmonic trap: 9 steps, so each psi array is
    read as the box, read as the previous-stage tile and written in turn."""
    tz, ty, idx = shape
    n = _grid_for(tz, ty, bc, zper)
    p = params(n=n, L=(0.5 * n[0], 0.5 * n[1], 0.5 * n[2]), prec=prec, bc=bc, periodicz=zper, pot="harmonic",
               harm=(40.0, 50.0, 60.0), omega=0.35, dt=0.01)
    psi = smooth_state(p, seed=23)
    s = Solver(p)
    s.set_kernel(2, -(idx + 1), 0)
    s.set_stage_form(abi.RK3_PSI_DIFF)
    assert s.stage_form() == abi.RK3_PSI_DIFF
    s.set_psi(psi)
    o = Oracle(p)
    o.set_psi(s.get_psi())
    s.step_rt(9)
    o.step_rt(9)
    a = s.get_psi().astype(np.complex128)
    b = o.get_psi().astype(np.complex128)
    if prec == abi.FP64:
        assert rel_err(a, b) < FP64_TOL
    else:
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-6
    d, do = s.diag(), o.diag()
    tol = FP64_TOL if prec == abi.FP64 else 2e-6
    for k in ("norm", "energy", "maxpsi", "intpsi2"):
        assert abs(d[k] - do[k]) <= tol * abs(do[k]), (k, d[k], do[k])
    assert abs(s.t - o.t) < 1e-14
    s.close()


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_psi_diff_partial_tiles_long_run(prec):
    """Grids that are not a multiple of the tile (zero ghosts from the TMA
    fill, partial previous-stage tiles) and 40 steps."""
    n = (9, 13, 70)
    p = params(n=n, L=(4.5, 6.5, 35.0), prec=prec, pot="harmonic", harm=(3.0, 4.0, 5.0), omega=0.2, dt=0.01)
    psi = smooth_state(p, seed=6)
    s = Solver(p)
    s.set_kernel(2, -1, 0)
    s.set_stage_form(abi.RK3_PSI_DIFF)
    assert s.stage_form() == abi.RK3_PSI_DIFF
    s.set_psi(psi)
    o = Oracle(p)
    o.set_psi(s.get_psi())
    s.step_rt(40)
    o.step_rt(40)
    a = s.get_psi().astype(np.complex128)
    b = o.get_psi().astype(np.complex128)
    if prec == abi.FP64:
        assert rel_err(a, b) < FP64_TOL
    else:
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 4e-6
    s.close()


@pytest.mark.parametrize("nproc", [(1, 1), (2, 2)])
def test_psi_diff_vortex_line_64_fp64_200_steps(nproc):
    """The 64^3 FP64 vortex-line workload (also on the 2 x 2 process-grid
    coordinates), 200 RK3 steps in the psi-difference form: psi, norm and
    energy to 1e-12 of the oracle's three-stage run."""
    prob, init = units.vortex_line_64(abi.FP64, nproc=nproc)
    p = prob.to_params()
    s = Solver(p)
    s.set_stage_form(abi.RK3_PSI_DIFF)
    s.init_state(init["name"], amp=init["amp"], r_tf2=init["r_tf2"], core2=init["core2"])
    assert s.stage_form() == abi.RK3_PSI_DIFF
    o = Oracle(p)
    o.set_psi(s.get_psi())
    s.step_rt(init["steps"])
    o.step_rt(init["steps"])
    a, b = s.get_psi(), o.get_psi()
    assert rel_err(a, b) < FP64_TOL
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < FP64_TOL
    dg, do = s.diag(), o.diag()
    for k in ("norm", "energy", "mu", "intpsi2", "maxpsi", "meanpsi"):
        assert abs(dg[k] - do[k]) <= FP64_TOL * abs(do[k]), (k, dg[k], do[k])
    assert abs(s.t - o.t) < 1e-14
    s.close()


def test_psi_diff_mixes_with_three_stages():
    """The state lives in the current psi array after every step, so forms can
    alternate between calls: 5 psi-difference + 5 three-stage + 5
    psi-difference steps in FP64 match 15 oracle steps."""
    n = (12, 16, 64)
    p = params(n=n, L=(6.0, 8.0, 32.0), prec=abi.FP64, pot="harmonic", harm=(3.0, 4.0, 5.0), omega=0.2, dt=0.01)
    psi = smooth_state(p, seed=11)
    s = Solver(p)
    s.set_psi(psi)
    o = Oracle(p)
    o.set_psi(s.get_psi())
    for form in (abi.RK3_PSI_DIFF, abi.RK3_THREE_STAGE, abi.RK3_PSI_DIFF):
        s.set_stage_form(form)
        s.step_rt(5)
    o.step_rt(15)
    assert rel_err(s.get_psi(), o.get_psi()) < FP64_TOL
    s.close()


def test_psi_diff_applicability():
    """Only on request, and only where the plain tiled stages run; elsewhere
    the step keeps three stages (and reports so)."""
    n = (12, 32, 128)
    base = dict(n=n, L=(6.0, 16.0, 64.0), pot="harmonic", harm=(3.0, 4.0, 5.0), dt=0.01)
    for prec in (abi.FP32, abi.FP64):
        s = Solver(params(prec=prec, omega=0.2, **base))
        assert s.stage_form() == abi.RK3_THREE_STAGE
        s.set_stage_form(abi.RK3_PSI_DIFF)
        assert s.stage_form() == abi.RK3_PSI_DIFF      # the default real-time shape
        s.set_kernel(1)                                 # per-cell kernel
        assert s.stage_form() == abi.RK3_THREE_STAGE
        s.close()
    s = Solver(params(prec=abi.FP32, vx=0.1, **base))
    s.set_stage_form(abi.RK3_PSI_DIFF)
    assert s.stage_form() == abi.RK3_THREE_STAGE       # advective frame: general variant
    s.close()
