"""Known-answer and restatement tests of the oracle's output-time diagnostics
(get_phase velocity and get_qpressure, diagnostic.f90:27-84), no GPU.

Pins: the velocity of a phase-modulated plane wave converges to the exact
phase gradient at 6th order, the quantum pressure of a smooth real density
to grad(lap rho) at 2nd order; and an independent numpy restatement built
from a globally padded array, cut into per-rank ghosted blocks whose edge
and corner ghosts are zero, agrees with the oracle for every boundary rule
and process grid.
"""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from trapbec_gb300 import abi
from tests.helpers import params, coords, smooth_state


def _plane_phase(n, a=1.0):
    L = 6.0
    p = params(n=(n, 8, 8), L=(L, 2.0, 2.0), bc=abi.BC_PERIODIC, periodicz=1)
    x, _, _ = coords(p)
    k = 2 * np.pi / L
    psi = np.exp(1j * a * np.sin(k * x))[:, None, None] * np.ones((n, 8, 8))
    exact = a * k * np.cos(k * x)
    return p, psi, exact


def test_velocity_sixth_order():
    errs = []
    for n in (24, 48):
        p, psi, exact = _plane_phase(n)
        o = Oracle(p)
        o.set_psi(psi)
        v = o.velocity()
        errs.append(np.max(np.abs(v[0] - exact[:, None, None])))
        assert np.max(np.abs(v[1])) < 1e-12 and np.max(np.abs(v[2])) < 1e-12
    assert errs[1] < 1e-7
    assert 45 < errs[0] / errs[1] < 90   # 2^6 = 64


def test_qpressure_second_order():
    """grad(lap rho) at 2nd order away from the domain edges.  laplace_rho on
    a ghost plane reads edge ghosts (zero) within two cells of a crossing
    face, so cells next to two faces at once carry that error, as in the
    reference; the comparison covers the cells clear of it."""
    errs = []
    L = 6.0
    for n in (32, 64):
        p = params(n=(n, 10, 10), L=(L, 2.5, 2.5), bc=abi.BC_PERIODIC, periodicz=1)
        x, _, _ = coords(p)
        k = 2 * np.pi / L
        psi = (2.0 + np.cos(k * x))[:, None, None] * np.ones((n, 10, 10)) + 0j
        o = Oracle(p)
        o.set_psi(psi)
        q = o.qpressure()
        exact = k ** 3 * np.sin(k * x)   # d/dx of -k^2 cos(kx)
        deep = (slice(None), slice(3, -3), slice(3, -3))
        errs.append(np.max(np.abs(q[0][deep] - exact[:, None, None])))
        assert np.max(np.abs(q[1][3:-3][deep])) < 1e-10 and np.max(np.abs(q[2][3:-3][deep])) < 1e-10
        # the edge-ghost zeros do show next to the faces
        assert np.max(np.abs(q[1][:, 0, :])) > 1.0
    assert 3.5 < errs[0] / errs[1] < 4.5


# ---- independent numpy restatement ---------------------------------------

def _global_pad(psi, p):
    """Ghost faces of the whole domain by the boundary rules (ghost.f90)."""
    modes = {abi.BC_PERIODIC: "wrap", abi.BC_SOLID: "reflect", abi.BC_ZERO: "constant"}
    bcz = abi.BC_PERIODIC if (p.periodicz or p.boundaries == abi.BC_PERIODIC) else p.boundaries
    g = psi
    for ax, bc in ((0, p.boundaries), (1, p.boundaries), (2, bcz)):
        pw = [(0, 0)] * 3
        pw[ax] = (3, 3)
        g = np.pad(g, pw, mode=modes[bc])
    return g


def _rank_blocks(psi, p):
    """(slices of the global interior, ghosted block with zero edges) per rank."""
    g = _global_pad(psi, p)
    nmx, nmy, nmz = p.nx // p.nprocx, p.ny // p.nprocy, p.nz
    out = []
    for cx in range(p.nprocx):
        for cy in range(p.nprocy):
            li, lj = cx * nmx, cy * nmy
            b = g[li:li + nmx + 6, lj:lj + nmy + 6, :].copy()
            ox = np.r_[np.ones(3), np.zeros(nmx), np.ones(3)].astype(int)
            oy = np.r_[np.ones(3), np.zeros(nmy), np.ones(3)].astype(int)
            oz = np.r_[np.ones(3), np.zeros(nmz), np.ones(3)].astype(int)
            outside = ox[:, None, None] + oy[None, :, None] + oz[None, None, :]
            b[outside > 1] = 0
            out.append(((slice(li, li + nmx), slice(lj, lj + nmy)), b))
    return out


def _d1(f, ax, h, lo, n):
    s = lambda m: np.take(f, range(lo + m, lo + m + n), axis=ax)
    return (-s(-3) + 9 * s(-2) - 45 * s(-1) + 45 * s(1) - 9 * s(2) + s(3)) / (60 * h)


def _np_velocity(psi, p):
    h = (p.lx / p.nx, p.ly / p.ny, p.lz / p.nz)
    v = np.zeros((3,) + psi.shape)
    for (sx, sy), b in _rank_blocks(psi, p):
        ph = np.arctan2(b.imag, b.real)
        nm = (b.shape[0] - 6, b.shape[1] - 6, b.shape[2] - 6)
        for c in range(3):
            d = _d1(ph, c, h[c], 3, nm[c])
            idx = [slice(3, 3 + nm[a]) if a != c else slice(None) for a in range(3)]
            v[c][sx, sy, :] = d[tuple(idx)]
    return v


def _np_qpressure(psi, p):
    h = (p.lx / p.nx, p.ly / p.ny, p.lz / p.nz)
    q = np.zeros((3,) + psi.shape)
    for (sx, sy), b in _rank_blocks(psi, p):
        den = np.abs(b)
        nm = (b.shape[0] - 6, b.shape[1] - 6, b.shape[2] - 6)
        # laplace_rho on local indices 0..n+1 = block indices 2..n+3
        cut = tuple(slice(2, 4 + nm[a]) for a in range(3))
        lap = np.zeros(tuple(nm[a] + 2 for a in range(3)))
        for c in range(3):
            s = lambda m: den[tuple(slice(2 + m, 4 + nm[a] + m) if a == c else cut[a] for a in range(3))]
            lap += (-s(-2) + 16 * s(-1) - 30 * s(0) + 16 * s(1) - s(2)) / (12 * h[c] ** 2)
        for c in range(3):
            s = lambda m: lap[tuple(slice(1 + m, 1 + nm[a] + m) if a == c else slice(1, 1 + nm[a])
                                    for a in range(3))]
            q[c][sx, sy, :] = (-s(-1) + s(1)) / (2 * h[c])
    return q


CASES = [(abi.BC_ZERO, 0, (1, 1)), (abi.BC_ZERO, 0, (2, 2)), (abi.BC_PERIODIC, 0, (1, 2)),
         (abi.BC_SOLID, 0, (2, 1)), (abi.BC_ZERO, 1, (2, 2)), (abi.BC_SOLID, 1, (1, 1))]


@pytest.mark.parametrize("bc,pz,nproc", CASES)
def test_diag_matches_numpy_restatement(bc, pz, nproc):
    p = params(n=(12, 16, 10), L=(6.0, 7.0, 5.0), bc=bc, periodicz=pz, nproc=nproc)
    rng = np.random.default_rng(11)
    psi = smooth_state(p, seed=4) + 0.05 * (rng.normal(size=(12, 16, 10)) + 1j * rng.normal(size=(12, 16, 10)))
    o = Oracle(p)
    o.set_psi(psi)
    v, q = o.velocity(), o.qpressure()
    vn, qn = _np_velocity(psi, p), _np_qpressure(psi, p)
    assert np.max(np.abs(v - vn)) <= 1e-12 * np.max(np.abs(vn))
    assert np.max(np.abs(q - qn)) <= 1e-12 * np.max(np.abs(qn))


def test_qpressure_depends_on_process_grid():
    """Edge ghosts are zero per rank: the quantum pressure next to a rank
    corner differs from the single-rank value; the velocity does not."""
    rng = np.random.default_rng(5)
    psi = 1.0 + 0.1 * (rng.normal(size=(12, 12, 8)) + 1j * rng.normal(size=(12, 12, 8)))
    res = {}
    for nproc in ((1, 1), (2, 2)):
        p = params(n=(12, 12, 8), L=(6.0, 6.0, 4.0), bc=abi.BC_PERIODIC, nproc=nproc)
        o = Oracle(p)
        o.set_psi(psi)
        res[nproc] = (o.velocity(), o.qpressure())
    assert np.max(np.abs(res[(1, 1)][0] - res[(2, 2)][0])) <= 1e-12
    dq = np.abs(res[(1, 1)][1] - res[(2, 2)][1])
    assert dq.max() > 1e-3
    # the difference lives within one cell of rank boundaries in x and y together
    far = dq[:, 2:4, 2:4, :]
    assert far.max() <= 1e-12


# ---- forcing (force.f90) ---------------------------------------------------

def test_force_vortex_oracle_known_answers():
    """psi = 1 forced at (x0, y0): |psi| = pade_density(r), which vanishes on
    the axis and tends to 1 far away; the phase winds by 2 pi dir around it;
    forcing +1 then -1 at the same point leaves pade_density(r)^2, real."""
    p = params(n=(48, 48, 4), L=(24.0, 24.0, 2.0), bc=abi.BC_PERIODIC, periodicz=1)
    x, y, _ = coords(p)
    x0, y0 = 0.37, -0.81
    for d in (1, -1):
        o = Oracle(p)
        o.set_psi(np.ones((48, 48, 4), dtype=np.complex128))
        o.force_vortex(x0, y0, d)
        ps = o.get_psi()[:, :, 0]
        r = np.hypot(x[:, None] - x0, y[None, :] - y0)
        assert np.abs(ps).min() < 0.3 and np.abs(np.abs(ps) - 1)[r > 10].max() < 1e-2
        # circulation along the square loop of cells 12..36
        loop = np.r_[ps[12:36, 12], ps[36, 12:36], ps[36:12:-1, 36], ps[12, 36:12:-1], ps[12, 12]]
        dphi = np.angle(loop[1:] / loop[:-1])
        assert abs(dphi.sum() - 2 * np.pi * d) < 1e-9
    o = Oracle(p)
    o.set_psi(np.ones((48, 48, 4), dtype=np.complex128))
    o.force_vortex(x0, y0, 1)
    a = o.get_psi().copy()
    o.force_vortex(x0, y0, -1)
    b = o.get_psi()
    assert np.abs(b.imag).max() < 1e-15
    assert np.allclose(b.real, np.abs(a) ** 2, rtol=0, atol=1e-14)
