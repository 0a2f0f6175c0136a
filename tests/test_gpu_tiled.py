"""The tiled (TMA) stage kernel against the CPU oracle and the per-cell kernel,
for every instantiated tile shape and boundary type, including partial tiles."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from trapbec_gb300 import Solver, abi
from tests.helpers import params, smooth_state, rel_err

pytestmark = pytest.mark.gpu

# built shapes by index (FP32: (128,8), (64,8), (64,16), (64,8) with 6 slots / 3 CTAs per SM, (64,32) with 4 rows per thread)
SHAPES = {abi.FP32: [(128, 8, 0), (64, 8, 1), (64, 16, 2), (64, 8, 3), (64, 32, 4)],
          abi.FP64: [(32, 8, 0), (64, 8, 1)]}


def _grid_for(tz, ty, bc, zper):
    # full tiles where the boundary needs fix-ups, two tiles per axis
    return (12, 2 * ty, 2 * tz)


def _shape_ids(v):
    return str(v)


CASES = [(prec, shp, bc, zper) for prec in (abi.FP64, abi.FP32) for shp in SHAPES[prec]
         for bc, zper in ((abi.BC_ZERO, 0), (abi.BC_SOLID, 0), (abi.BC_PERIODIC, 0), (abi.BC_ZERO, 1))]


@pytest.mark.parametrize("prec,shape,bc,zper", CASES, ids=lambda v: str(v))
def test_tiled_matches_oracle(prec, shape, bc, zper):
    tz, ty, idx = shape
    n = _grid_for(tz, ty, bc, zper)
    p = params(n=n, L=(0.5 * n[0], 0.5 * n[1], 0.5 * n[2]), prec=prec, bc=bc, periodicz=zper, pot="harmonic",
               harm=(40.0, 50.0, 60.0), omega=0.35, dt=0.01)
    psi = smooth_state(p, seed=21)
    s = Solver(p)
    s.set_kernel(2, -(idx + 1), 0)
    s.set_psi(psi)
    o = Oracle(p)
    o.set_psi(s.get_psi())
    tol_rhs = 1e-13 if prec == abi.FP64 else 3e-6
    assert rel_err(s.get_rhs(), o.get_rhs()) < tol_rhs
    s.step_rt(6)
    o.step_rt(6)
    a = s.get_psi().astype(np.complex128)
    b = o.get_psi().astype(np.complex128)
    if prec == abi.FP64:
        assert rel_err(a, b) < 1e-12
    else:
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-6
    d, do = s.diag(), o.diag()
    tol = 1e-12 if prec == abi.FP64 else 2e-6
    for k in ("norm", "energy", "maxpsi", "intpsi2"):
        assert abs(d[k] - do[k]) <= tol * abs(do[k]), (k, d[k], do[k])


@pytest.mark.parametrize("prec", [abi.FP32, abi.FP64])
def test_tiled_partial_tiles_zero_ghosts(prec):
    """Grids that are not a multiple of the tile: zero ghosts come from the
    TMA out-of-bounds fill, outputs beyond the grid are masked."""
    n = (9, 13, 70)
    p = params(n=n, L=(4.5, 6.5, 35.0), prec=prec, pot="harmonic", harm=(3.0, 4.0, 5.0), omega=0.2, dt=0.01)
    psi = smooth_state(p, seed=4)
    s, o = Solver(p), Oracle(p)
    s.set_kernel(2)
    s.set_psi(psi)
    o.set_psi(s.get_psi())
    s.step_rt(5)
    o.step_rt(5)
    a, b = s.get_psi().astype(np.complex128), o.get_psi().astype(np.complex128)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < (1e-13 if prec == abi.FP64 else 2e-6)


def test_tiled_equals_simple_fp32_array_potential():
    n = (10, 16, 64)
    p = params(n=n, L=(10.0, 16.0, 64.0), prec=abi.FP32, pot="array", vx=0.1, dt=0.01)
    trap = np.random.default_rng(2).uniform(0, 1, size=n)
    psi = smooth_state(p, seed=5)
    out = []
    for kind in (1, 2):
        s = Solver(p)
        s.set_kernel(kind)
        s.set_trap(trap)
        s.set_psi(psi)
        s.step_rt(4)
        out.append(s.get_psi().astype(np.complex128))
    assert np.linalg.norm(out[0] - out[1]) / np.linalg.norm(out[1]) < 1e-6


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_tiled_imag_rk3(prec):
    n = (16, 16, 64)
    p = params(n=n, L=(8.0, 8.0, 16.0), prec=prec, pot="harmonic", harm=(64.0, 64.0, 256.0), omega=0.3, dt=0.005)
    psi = smooth_state(p, seed=8)
    s, o = Solver(p), Oracle(p)
    s.set_kernel(2)
    s.set_psi(psi)
    o.set_psi(s.get_psi())
    sg, _ = s.step_imag(60, abi.IMAG_RK3_RENORM, 0.0)
    so, _ = o.step_imag_rk3(60, 0.0)
    assert sg == so == 60
    a, b = s.get_psi().astype(np.complex128), o.get_psi().astype(np.complex128)
    d, do = s.diag(), o.diag()
    if prec == abi.FP64:
        assert rel_err(a, b) < 1e-11
        assert abs(d["energy"] - do["energy"]) < 1e-12 * abs(do["energy"])
    else:
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-5
        assert abs(d["energy"] - do["energy"]) < 1e-5 * abs(do["energy"])
    assert abs(d["norm"] / do["norm"] - 1) < (1e-12 if prec == abi.FP64 else 1e-6)


DEFER_CASES = [(shp, bc, zper) for shp in SHAPES[abi.FP32]
               for bc, zper in ((abi.BC_ZERO, 0), (abi.BC_SOLID, 0), (abi.BC_PERIODIC, 0), (abi.BC_ZERO, 1))]
DEFER_SHAPES = (0, 1, 2)   # shapes whose shared memory holds the deferred stage's two boxes per slot


@pytest.mark.parametrize("shape,bc,zper", DEFER_CASES, ids=lambda v: str(v))
def test_deferred_form_bitwise_equals_three_stages(shape, bc, zper):
    """The deferred real-time form (stage 1 stores w1 only, stage 2 forms
    psi1 = psi0 + w1/3 from ghosted boxes of psi0 and w1) gives the same bits
    as three full stages, including the ghost fix-ups of boundary tiles."""
    tz, ty, idx = shape
    n = _grid_for(tz, ty, bc, zper)
    p = params(n=n, L=(0.5 * n[0], 0.5 * n[1], 0.5 * n[2]), prec=abi.FP32, bc=bc, periodicz=zper, pot="harmonic",
               harm=(40.0, 50.0, 60.0), omega=0.35, dt=0.01)
    psi = smooth_state(p, seed=31)
    out = []
    for form in (abi.RK3_DEFERRED, abi.RK3_THREE_STAGE):
        s = Solver(p)
        s.set_kernel(2, -(idx + 1), 0)
        s.set_stage_form(form)
        assert s.stage_form_deferred() == (form == abi.RK3_DEFERRED and idx in DEFER_SHAPES)
        s.set_psi(psi)
        s.step_rt(7)
        out.append(s.get_psi())
        s.close()
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


def test_deferred_form_partial_tiles_and_long_run():
    """Partial tiles (zero ghosts from the TMA fill) and many steps, so both w
    buffers are reused across steps."""
    n = (9, 13, 70)
    p = params(n=n, L=(4.5, 6.5, 35.0), prec=abi.FP32, pot="harmonic", harm=(3.0, 4.0, 5.0), omega=0.2, dt=0.01)
    psi = smooth_state(p, seed=6)
    out = []
    for form in (abi.RK3_DEFERRED, abi.RK3_THREE_STAGE):
        s = Solver(p)
        s.set_kernel(2, -1, 0)
        s.set_stage_form(form)
        assert s.stage_form_deferred() == (form == abi.RK3_DEFERRED)
        s.set_psi(psi)
        s.step_rt(40)
        out.append(s.get_psi())
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


def test_deferred_form_applicability():
    """Three stages by default; deferred only on request, where the plain FP32
    tiled stages run on a shape that holds its boxes."""
    n = (12, 32, 128)
    base = dict(n=n, L=(6.0, 16.0, 64.0), pot="harmonic", harm=(3.0, 4.0, 5.0), dt=0.01)
    s = Solver(params(prec=abi.FP32, omega=0.2, **base))
    assert not s.stage_form_deferred()
    s.set_stage_form(abi.RK3_DEFERRED)
    assert not s.stage_form_deferred()   # the default real-time shape (64 x 32) cannot hold both boxes
    s.set_kernel(2, -1, 0)               # shape 0 for every launch
    assert s.stage_form_deferred()
    s.set_kernel(1)                      # per-cell kernel
    assert not s.stage_form_deferred()
    s.close()
    s = Solver(params(prec=abi.FP64, **base))
    s.set_stage_form(abi.RK3_DEFERRED)
    assert not s.stage_form_deferred()
    s = Solver(params(prec=abi.FP32, vx=0.1, **base))
    s.set_stage_form(abi.RK3_DEFERRED)
    s.set_kernel(2, -1, 0)
    assert not s.stage_form_deferred()   # advective frame: general variant


def test_real_time_shape_equals_general_shape():
    """The default plan split (64 x 32 tiles for the plain real-time stages,
    shape 0 for the rest) against shape 0 everywhere: same bits."""
    n = (20, 64, 128)
    p = params(n=n, L=(10.0, 32.0, 64.0), prec=abi.FP32, bc=abi.BC_SOLID, pot="harmonic", harm=(3.0, 4.0, 5.0),
               omega=0.3, dt=0.01)
    psi = smooth_state(p, seed=12)
    out = []
    for explicit in (False, True):
        s = Solver(p)
        if explicit:
            s.set_kernel(2, -1, 0)
        s.set_psi(psi)
        s.step_rt(9)
        out.append((s.get_psi(), s.diag()["energy"]))
    assert np.array_equal(out[0][0].view(np.uint32), out[1][0].view(np.uint32))
    assert out[0][1] == out[1][1]


IMAG_VARIANT_CASES = [("harmonic", 0.3, 0.0), ("zero", 0.0, 0.0), ("array", 0.2, 0.0), ("harmonic", 0.0, 0.15)]


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
@pytest.mark.parametrize("pot,omega,vx", IMAG_VARIANT_CASES, ids=lambda v: str(v))
def test_tiled_imag_rk3_variants(prec, pot, omega, vx):
    """Imaginary-time RK3 through both kernel variants against the oracle:
    harmonic / no potential with rotation / no frame take the imaginary-time
    variant, an array potential or the advective frame the general one."""
    n = (12, 16, 64)
    p = params(n=n, L=(6.0, 8.0, 32.0), prec=prec, pot="harmonic" if pot == "harmonic" else pot,
               harm=(40.0, 50.0, 60.0), omega=omega, vx=vx, dt=0.005)
    psi = smooth_state(p, seed=17)
    s, o = Solver(p), Oracle(p)
    s.set_kernel(2)
    if pot == "array":
        trap = np.random.default_rng(5).uniform(0, 1, size=n)
        s.set_trap(trap)
        o.set_trap(trap)
    s.set_psi(psi)
    o.set_psi(s.get_psi())
    sg, _ = s.step_imag(80, abi.IMAG_RK3_RENORM, 0.0)
    so, _ = o.step_imag_rk3(80, 0.0)
    assert sg == so == 80
    a, b = s.get_psi().astype(np.complex128), o.get_psi().astype(np.complex128)
    d, do = s.diag(), o.diag()
    if prec == abi.FP64:
        assert rel_err(a, b) < 1e-11
        assert abs(d["energy"] - do["energy"]) < 1e-12 * abs(do["energy"])
    else:
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-5
        assert abs(d["energy"] - do["energy"]) < 1e-5 * abs(do["energy"])


def test_default_plan_falls_back_to_a_shape_that_fits():
    """Solid walls need whole tiles: at nz = 64 the (128 x 8) shape cannot
    plan, so the default plans take the first built shape that does (64 x 8)
    instead of the per-cell kernel; results still match the oracle."""
    n = (12, 16, 64)
    p = params(n=n, L=(6.0, 8.0, 32.0), prec=abi.FP32, bc=abi.BC_SOLID, pot="harmonic", harm=(40.0, 50.0, 60.0),
               omega=0.3, dt=0.01)
    psi = smooth_state(p, seed=23)
    s, o = Solver(p), Oracle(p)
    assert s.tile_shape(real_time=False) == (64, 8)
    assert s.tile_shape(real_time=True) == (64, 8)    # (64 x 32) needs ny divisible by 32 with solid walls
    s.set_psi(psi)
    o.set_psi(s.get_psi())
    s.step_rt(6)
    o.step_rt(6)
    a, b = s.get_psi().astype(np.complex128), o.get_psi().astype(np.complex128)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-6


@pytest.mark.parametrize("prec", [abi.FP32, abi.FP64])
@pytest.mark.parametrize("form", [abi.RK3_THREE_STAGE, abi.RK3_PSI_DIFF])
@pytest.mark.parametrize("chunk", [-8, -36, -128])
def test_strided_order_gives_the_same_states(prec, form, chunk):
    """The strided work order (set_chunk < 0: segments dealt round-robin over
    the CTAs) changes which CTA streams which tiles and x-range, not the
    arithmetic of a point: the states are bit for bit those of the default
    order.  96 x 128 x 256 has 16 tiles of (64 x 32): chunks of 8 planes make
    192 segments (more than the CTAs), of 36 a ragged last chunk and idle
    CTAs, of 128 (clamped to nx) one segment per tile.  The diagnostics run
    in the same order, with their partial sums grouped by CTA differently."""
    p = params(n=(96, 128, 256), L=(24.0, 32.0, 64.0), prec=prec, pot="harmonic", harm=(3.0, 4.0, 5.0),
               omega=0.3, dt=0.01)
    psi = smooth_state(p, seed=31)
    out = {}
    for ch in (0, chunk):
        s = Solver(p)
        s.set_stage_form(form)
        s.set_chunk(ch)
        s.set_psi(psi)
        s.step_rt(6)
        out[ch] = (s.get_psi(), s.diag())
        s.close()
    (a, da), (b, db) = out[0], out[chunk]
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    for k in ("intpsi2", "energy", "maxpsi", "minpsi"):
        assert abs(da[k] - db[k]) <= 1e-9 * abs(da[k]), (k, da[k], db[k])
