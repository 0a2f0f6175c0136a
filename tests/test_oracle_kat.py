"""Known-answer tests that pin the CPU oracle (no GPU).

The reference cannot be built here and ships no golden vectors, so the
oracle's restatement of the hot path is pinned by mathematics: stencil
exactness on polynomials and the 6th-order convergence slope, the Lz
eigenvalue of x+iy, the RK3 stability polynomial, norm conservation, the
harmonic-oscillator ground state, and the equivalence of a 2x2 virtual
process grid with one rank.
"""
import json
import os
from fractions import Fraction

import numpy as np
import pytest

from oracle.pyoracle import Oracle
from trapbec_gb300 import abi
from tests.helpers import params, coords, smooth_state, rel_err

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _interior(a, m=3):
    return a[m:-m, m:-m, m:-m]


def _nonlin(psi, pot=0.0):
    # (1 - abs(Psi**2) - pot) * Psi  (finite_diff.f90:132)
    return (1.0 - np.abs(psi * psi) - pot) * psi


def test_stencil_golden_exact_rationals():
    """The golden file holds exact stencil values; D2 is exact to degree 7, D1 to 6."""
    g = json.load(open(os.path.join(GOLD, "kat_stencils.json")))
    for e in g["d2"]:
        if e["n"] <= 7:
            assert Fraction(e["stencil"]) == Fraction(e["exact"]), e
        else:
            assert Fraction(e["stencil"]) != Fraction(e["exact"]), e
    for e in g["d1"]:
        if e["n"] <= 6:
            assert Fraction(e["stencil"]) == Fraction(e["exact"]), e
    # symbol at theta = pi: (2*2*(-1) - 27*2 + 270*2*(-1) - 490)/180 = -1088/180
    assert abs(g["d2_symbol_at"]["pi"] + 1088 / 180) < 1e-12


@pytest.mark.parametrize("prec,tol", [(abi.FP64, 1e-9), (abi.FP32, 2e-3)])
def test_d2_exact_on_polynomials(prec, tol):
    """get_rhs on psi = eps*p(x), deg p = 7, equals eps*p'' + nonlinear term."""
    p = params(n=(24, 8, 8), L=(6.0, 2.0, 2.0), prec=prec, bc=abi.BC_PERIODIC, periodicz=1)
    x, y, z = coords(p)
    rng = np.random.default_rng(3)
    c = rng.normal(size=8) + 1j * rng.normal(size=8)
    poly = np.polynomial.Polynomial(c)
    eps = 1e-3
    X = np.broadcast_to(x[:, None, None], (24, 8, 8)) / 3.0
    psi = eps * poly(X)
    o = Oracle(p)
    o.set_psi(psi)
    rhs = o.get_rhs()
    exact = eps * poly.deriv(2)(X) / 9.0 + _nonlin(o.get_psi().astype(np.complex128))
    sl = (slice(3, -3), slice(None), slice(None))  # x-interior; y/z periodic and constant
    assert rel_err(rhs[sl], exact[sl]) < tol


def test_d2_sixth_order_convergence():
    errs = []
    for n in (32, 64):
        p = params(n=(n, 4, 4), L=(2 * np.pi, 1.0, 1.0), bc=abi.BC_PERIODIC, periodicz=1)
        x, _, _ = coords(p)
        eps = 1e-6
        psi = eps * np.exp(3j * x)[:, None, None] * np.ones((1, 4, 4))
        o = Oracle(p)
        o.set_psi(psi)
        rhs = o.get_rhs()
        lap = rhs - _nonlin(o.get_psi())
        errs.append(np.max(np.abs(lap - (-9.0) * psi)) / eps)
    order = np.log2(errs[0] / errs[1])
    assert 5.8 < order < 6.2, (errs, order)


def test_rotation_term_lz_eigenvalue():
    """psi = eps (x + i y): D1 is exact, Lz psi = psi, so the rotation term of
    get_rhs is omega*i*(x*i - y) = -omega*psi (finite_diff.f90:128-131)."""
    om = 0.37
    p = params(n=(16, 16, 8), L=(4.0, 4.0, 2.0), omega=om, bc=abi.BC_ZERO)
    x, y, z = coords(p)
    eps = 1e-4
    psi = eps * (x[:, None, None] + 1j * y[None, :, None]) * np.ones((1, 1, 8))
    o = Oracle(p)
    o.set_psi(psi)
    rhs = o.get_rhs()
    expect = -om * psi + _nonlin(psi)
    # z has zero ghosts: take a z-independent comparison away from z and xy edges
    sl = (slice(3, -3), slice(3, -3), slice(3, 5))
    lapz = np.zeros_like(psi)  # psi constant in z on the interior slice: D2z = 0 there
    assert rel_err(rhs[sl], (expect + lapz)[sl]) < 1e-10


def test_advective_term():
    """psi = eps*e^{i k x}: 2*i*vx*D1x psi = 2*i*vx*(i k~) psi (k~ the D1 symbol)."""
    vx = 0.25
    n = 32
    p = params(n=(n, 4, 4), L=(2 * np.pi, 1.0, 1.0), vx=vx, bc=abi.BC_PERIODIC, periodicz=1)
    x, _, _ = coords(p)
    h = 2 * np.pi / n
    k = 2.0
    eps = 1e-6
    psi = eps * np.exp(1j * k * x)[:, None, None] * np.ones((1, 4, 4))
    o = Oracle(p)
    o.set_psi(psi)
    rhs = o.get_rhs()
    th = k * h
    d1sym = (2 * np.sin(3 * th) * 1 - 9 * 2 * np.sin(2 * th) + 45 * 2 * np.sin(th)) / (60 * h)
    d2sym = (2 * 2 * np.cos(3 * th) - 27 * 2 * np.cos(2 * th) + 270 * 2 * np.cos(th) - 490) / (180 * h * h)
    expect = d2sym * psi + 2j * vx * (1j * d1sym) * psi + _nonlin(psi)
    assert rel_err(rhs, expect) < 1e-9


def test_rk3_stability_polynomial():
    g = json.load(open(os.path.join(GOLD, "kat_rk3.json")))
    assert g["coeffs"] == ["1", "1", "1/2", "1/6", "0"]
    # One real-time step of a tiny constant state in a periodic box with no
    # potential: rhs = (1 - |psi|^2) psi ~ psi, so psi1/psi0 = R(i dt/2).
    dt = 0.3
    p = params(n=(8, 8, 8), L=(4.0, 4.0, 4.0), bc=abi.BC_PERIODIC, periodicz=1, dt=dt)
    o = Oracle(p)
    eps = 1e-9
    o.set_psi(np.full((8, 8, 8), eps * (0.6 + 0.8j)))
    o.step_rt(1)
    ratio = o.get_psi()[3, 3, 3] / (eps * (0.6 + 0.8j))
    zz = 0.5j * dt
    R = 1 + zz + zz ** 2 / 2 + zz ** 3 / 6
    assert abs(ratio - R) < 1e-13
    for re, im, vr, vi in g["values"]:
        zc = complex(re, im)
        assert abs(1 + zc + zc ** 2 / 2 + zc ** 3 / 6 - complex(vr, vi)) < 1e-14


def test_norm_conservation_real_time():
    p = params(n=(24, 24, 24), L=(12.0, 12.0, 12.0), pot="harmonic", harm=(30.0, 30.0, 30.0), dt=0.01,
               omega=0.2)
    o = Oracle(p)
    o.set_psi(smooth_state(p, seed=1))
    n0 = o.diag()["norm"]
    e0 = o.diag()["energy"]
    o.step_rt(50)
    d = o.diag()
    assert abs(d["norm"] / n0 - 1) < 1e-6
    assert abs(d["energy"] / e0 - 1) < 1e-5


def test_harmonic_oscillator_ground_state():
    """Linear limit (tiny norm): imaginary-time RK3 + renormalisation relaxes to
    the HO ground state, mu = sum(Omega_a)/2 with Omega_a = sqrt(harm_w_a)/L_a;
    the discretisation error falls at 6th order under refinement."""
    L = 10.0
    om = (1.0, 1.3, 0.8)
    harm = tuple((w * L) ** 2 for w in om)
    errs = []
    for n in (24, 32):
        p = params(n=(n, n, n), L=(L, L, L), pot="harmonic", harm=harm, dt=0.02 * (24 / n) ** 2)
        o = Oracle(p)
        x, y, z = coords(p)
        g = np.exp(-0.3 * (x[:, None, None] ** 2 + y[None, :, None] ** 2 + z[None, None, :] ** 2))
        o.set_psi(1e-6 * g.astype(np.complex128))
        n0 = o.diag()["norm"]
        steps, rel = o.step_imag_rk3(20000, 1e-13)
        d = o.diag()
        assert rel <= 1e-13 and steps < 20000
        assert abs(d["norm"] / n0 - 1) < 1e-13  # renormalised to the initial norm
        errs.append(abs(d["mu"] - 0.5 * sum(om)))
    assert errs[1] < 3e-5
    assert errs[0] / errs[1] > 0.8 * (32 / 24) ** 6


@pytest.mark.parametrize("bc", [abi.BC_ZERO, abi.BC_SOLID, abi.BC_PERIODIC])
def test_virtual_ranks_match_single_rank(bc):
    """The 2x2 process grid (face exchange of ghost.f90) gives the single-rank
    result up to the rounding of its coordinates (initial.f90:38-41)."""
    base = dict(n=(16, 16, 12), L=(8.0, 8.0, 6.0), pot="harmonic", harm=(5.0, 6.0, 7.0), omega=0.4, bc=bc,
                dt=0.01)
    p1 = params(**base)
    p4 = params(nproc=(2, 2), **base)
    psi = smooth_state(p1, seed=5)
    o1, o4 = Oracle(p1), Oracle(p4)
    o1.set_psi(psi)
    o4.set_psi(psi)
    x1 = np.array(o1.coords()[0])
    x4 = np.array(o4.coords()[0])
    assert np.max(np.abs(x1 - x4)) < 1e-14
    o1.step_rt(10)
    o4.step_rt(10)
    assert rel_err(o4.get_psi(), o1.get_psi()) < 1e-12


def test_imag_euler_ratio():
    p = params(n=(12, 12, 12), L=(6.0, 6.0, 6.0), pot="harmonic", harm=(3.0, 3.0, 3.0), dt=0.01)
    o = Oracle(p)
    o.set_psi(smooth_state(p, seed=2))
    n0 = o.psi_norm_ref()
    r = o.step_imag_euler(1)
    n1 = o.psi_norm_ref()
    assert abs(r - n1 / 1.0) < 1e-12 * n1  # intPsi2_old starts at 1 (diagnostic.f90:5)
    r2 = o.step_imag_euler(1)
    assert abs(r2 - o.psi_norm_ref() / n1) < 1e-12
    assert n0 > 0


def test_oracle_regression_fixture():
    g = json.load(open(os.path.join(GOLD, "oracle_regress.json")))
    p = params(n=(12, 12, 12), L=(6.0, 6.0, 6.0), pot="harmonic", harm=tuple(g["harm"]), omega=g["omega"],
               dt=g["dt"])
    o = Oracle(p)
    o.set_psi(smooth_state(p, seed=g["seed"]))
    o.step_rt(g["steps"])
    a = o.get_psi()
    assert abs(a.real.sum() - g["sum_re"]) < 1e-12 * abs(g["sum_re"])
    assert abs(a.imag.sum() - g["sum_im"]) < 1e-10 * abs(g["sum_re"])
    assert abs((np.abs(a) ** 2).sum() - g["sum_abs2"]) < 1e-12 * g["sum_abs2"]
    assert abs(complex(*g["psi_mid"]) - a[6, 5, 4]) < 1e-14
    d = o.diag()
    assert abs(d["energy"] - g["energy"]) < 1e-12 * abs(g["energy"])


def test_ghost_fill_layout():
    """Ghost shell after ghost_comm for 'solid' x/y and periodic z."""
    p = params(n=(8, 8, 8), L=(4.0, 4.0, 4.0), bc=abi.BC_SOLID, periodicz=1)
    o = Oracle(p)
    psi = smooth_state(p, seed=4)
    o.set_psi(psi)
    g = o.get_psi_ghosted()  # (-2:n+3) per axis, C order (x, y, z)
    I = g[3:-3, 3:-3, 3:-3]
    assert np.array_equal(I, psi)
    # solid x: Psi(0)=Psi(2), Psi(-1)=Psi(3), Psi(-2)=Psi(4); 1-based -> offset +2
    for m in range(3):
        assert np.array_equal(g[2 - m, 3:-3, 3:-3], psi[1 + m])
        assert np.array_equal(g[8 + 3 + m, 3:-3, 3:-3], psi[8 - 2 - m])
    # periodic z: Psi(n+1)=Psi(1), Psi(0)=Psi(n)
    assert np.array_equal(g[3:-3, 3:-3, 11], psi[:, :, 0])
    assert np.array_equal(g[3:-3, 3:-3, 2], psi[:, :, 7])
