"""Map a Gross-Pitaevskii problem in "trap units" onto the reference's units.

Trap units:       i d(phi)/dt = -1/2 lap(phi) + V phi + g|phi|^2 phi - mu phi - Omega Lz phi,
                  V = 1/2 sum_a omega_a^2 x_a^2,  Lz = -i (x d_y - y d_x).
Reference units:  i d(psi)/dt' = -1/2 lap' psi + 1/2 (pot + |psi|^2 - 1) psi
                                 - 1/2 omega_z i (x' d_y' - y' d_x') psi
                  (finite_diff.f90:23-27,128-132 with run.f90:47: dpsi = i*0.5*dt*rhs).

With a = 1/sqrt(2 mu):  x = a x',  t = a^2 t',  phi = sqrt(mu/g) psi, so
  pot(x') = V(a x')/mu,  L' = L/a,  dt' = dt/a^2 = 2 mu dt,
  omega_z = -Omega/mu,
  harmonic: harm_w_a * (x'/L'_a)^2 = omega_a^2 x'^2 / (4 mu^2)
            => harm_w_a = omega_a^2 L'_a^2 / (4 mu^2),
  norms:    int |phi|^2 d^3x = (mu/g) a^3 int |psi|^2 d^3x',
  energies: E_trap = (mu/g) a^3 * 2 mu * E_ref  (E_ref as returned by
            trapbec_diag: dV' sum[-1/2 Re psi* lap + 1/2 pot |psi|^2
            + 1/4 |psi|^4 - 1/2 Re psi* rot]),
  chemical potential: mu_trap = 2 mu * mu_ref.

The reference's harmonic potential is the only trap shape the workloads use
(finite_diff.f90:33-34).
"""
from __future__ import annotations

import math

import numpy as np
from dataclasses import dataclass, field

from .abi import (Params, default_params, BC_ZERO, POT_HARMONIC, FP32, FP64)


@dataclass
class TrapProblem:
    """A GP problem in trap units on the cube [-L/2, L/2]^3 (cell-centred grid)."""

    n: tuple[int, int, int]          # (Nx, Ny, Nz)
    box: tuple[float, float, float]  # (Lx, Ly, Lz)
    omega: tuple[float, float, float]
    g: float
    mu: float                        # sets the unit scale (TF chemical potential)
    dt: float                        # real time step (or imaginary step)
    Omega: float = 0.0               # rotation, enters as -Omega Lz
    gamma: float = 0.0
    precision: int = FP64
    boundaries: int = BC_ZERO
    nproc: tuple[int, int] = (1, 1)

    @property
    def a(self) -> float:
        return 1.0 / math.sqrt(2.0 * self.mu)

    def to_params(self) -> Params:
        p = default_params()
        p.nx, p.ny, p.nz = self.n
        p.nprocx, p.nprocy = self.nproc
        p.precision = self.precision
        p.boundaries = self.boundaries
        p.periodicz = 0
        p.two_dim = 0
        p.potential = POT_HARMONIC
        a = self.a
        p.lx, p.ly, p.lz = (L / a for L in self.box)
        mu = self.mu
        p.harm_wx = self.omega[0] ** 2 * p.lx ** 2 / (4 * mu * mu)
        p.harm_wy = self.omega[1] ** 2 * p.ly ** 2 / (4 * mu * mu)
        p.harm_wz = self.omega[2] ** 2 * p.lz ** 2 / (4 * mu * mu)
        p.dt_re, p.dt_im = 2.0 * mu * self.dt, 0.0
        p.gamma = self.gamma
        p.omega_z = -self.Omega / mu
        return p

    # conversions of results back to trap units
    def psi_scale(self) -> float:
        """phi = psi_scale * psi."""
        return math.sqrt(self.mu / self.g)

    def norm_to_trap(self, norm_ref: float) -> float:
        return (self.mu / self.g) * self.a ** 3 * norm_ref

    def norm_to_ref(self, norm_trap: float) -> float:
        return norm_trap / ((self.mu / self.g) * self.a ** 3)

    def energy_to_trap(self, e_ref: float) -> float:
        return (self.mu / self.g) * self.a ** 3 * 2.0 * self.mu * e_ref

    def mu_to_trap(self, mu_ref: float) -> float:
        return 2.0 * self.mu * mu_ref

    def omega_z_for(self, Omega: float) -> float:
        return -Omega / self.mu

    def length_to_ref(self, x: float) -> float:
        return x / self.a

    def inv_r2_ref(self, R_trap: tuple[float, float, float]) -> list[float]:
        """1/R'^2 per axis in reference coordinates for TF radii R (trap units)."""
        return [(self.a / R) ** 2 for R in R_trap]


def tf_mu(omega: tuple[float, float, float], g: float, N: float) -> float:
    """Thomas-Fermi chemical potential for N atoms: mu = (15 g N w^3 / (8 pi sqrt(2)... ))

    From N = (8 pi / 15) (2 mu)^{3/2} mu / (g w_x w_y w_z) (TF integral of
    (mu - V)/g over the ellipsoid)."""
    wbar3 = omega[0] * omega[1] * omega[2]
    # N = 8*pi/15 * (2mu)^(3/2) * mu / (g * wbar3)  ->  mu^(5/2) = 15 g wbar3 N / (8 pi 2^(3/2))
    return (15.0 * g * wbar3 * N / (8.0 * math.pi * 2.0 ** 1.5)) ** 0.4


def tf_norm(omega: tuple[float, float, float], g: float, mu: float) -> float:
    wbar3 = omega[0] * omega[1] * omega[2]
    return 8.0 * math.pi / 15.0 * (2.0 * mu) ** 1.5 * mu / (g * wbar3)


# ---- the workload set ---------------------------------------------------------

def vortex_line_64(precision: int = FP64, nproc=(1, 1)) -> tuple[TrapProblem, dict]:
    """64^3 on [-16,16]^3 (dx = 0.5), isotropic omega = 0.1, g = 1, R_TF = 12,
    TF x Pade vortex line along z, RK3 dt = 0.005 for 200 steps."""
    w = 0.1
    R = 12.0
    mu = 0.5 * w * w * R * R  # 0.72
    prob = TrapProblem(n=(64, 64, 64), box=(32.0, 32.0, 32.0), omega=(w, w, w), g=1.0,
                       mu=mu, dt=0.005, precision=precision, nproc=nproc)
    a = prob.a
    # psi0(trap) = sqrt(max(0, 1 - r^2/R^2)) * rho/sqrt(rho^2 + 2) * e^{i theta};
    # in reference units psi = phi / sqrt(mu/g), rho = a rho'.
    init = dict(name="tf_vortex_line",
                amp=1.0 / prob.psi_scale(),
                r_tf2=[(a / R) ** 2] * 3,
                core2=2.0 / (a * a), steps=200)
    return prob, init


def vortex_ring_256(precision: int = FP64, n: int = 256, seed: int = 1234) -> tuple[TrapProblem, dict]:
    """256^3 on [-32,32]^3, omega = (0.05, 0.05, 0.1), g = 1, TF background x
    vortex ring of radius 8 in z = 0, phase noise 1e-3; RK3 dt = 0.005, 2000 steps.
    The TF radii follow from mu; mu is set by requiring the TF cloud to fill
    R_perp = 24 (0.75 of the half box)."""
    w = (0.05, 0.05, 0.1)
    Rperp = 24.0
    mu = 0.5 * w[0] ** 2 * Rperp ** 2  # 0.72
    L = 64.0
    prob = TrapProblem(n=(n, n, n), box=(L, L, L), omega=w, g=1.0, mu=mu, dt=0.005,
                       precision=precision)
    a = prob.a
    R = [math.sqrt(2 * mu) / wa for wa in w]
    init = dict(name="tf_vortex_ring", amp=1.0, r_tf2=[(a / Ra) ** 2 for Ra in R],
                ring_radius=8.0 / a, noise_amp=1e-3, seed=seed, steps=2000)
    return prob, init


def rotating_quench_512(precision: int = FP32, n: int = 512, seed: int = 99) -> tuple[TrapProblem, dict]:
    """512^3 on [-64,64]^3, omega_perp = 0.02, omega_z = 0.04, g = 1, dt = 0.004,
    Omega ramped 0 -> 0.8 omega_perp over 5000 steps.  Starts from a TF cloud
    with 1e-2 noise (standing in for a relaxed ground state) filling R_perp = 48."""
    wp, wz = 0.02, 0.04
    Rperp = 48.0
    mu = 0.5 * wp * wp * Rperp ** 2  # 0.4608
    L = 128.0
    prob = TrapProblem(n=(n, n, n), box=(L, L, L), omega=(wp, wp, wz), g=1.0, mu=mu,
                       dt=0.004, Omega=0.0, precision=precision)
    a = prob.a
    R = [math.sqrt(2 * mu) / wa for wa in (wp, wp, wz)]
    init = dict(name="tf_noise", amp=1.0, r_tf2=[(a / Ra) ** 2 for Ra in R],
                noise_amp=1e-2, seed=seed, steps=5000, omega_final=0.8 * wp)
    return prob, init


def ground_state_draws(count: int, seed: int, grids=(64, 96, 128), precision: int = FP32,
                       dtau: float = 0.002, res: float = 1.2) -> list[tuple[TrapProblem, dict]]:
    """Seeded parameter draws of the batched ground-state workload.

    omega_perp ~ U[0.05, 0.2], omega_z / omega_perp ~ U[0.5, 4], g log-uniform
    in [1, 1000], Omega ~ U[0, 0.7 omega_perp] (entering as -Omega Lz), grid
    uniform over `grids` (cubic in cells, box per axis 2.6 x the TF radius).
    The atom number is set so that the chemical potential keeps the healing
    length resolved: mu = res-scaled so that dx_perp ~ 1.2 xi.  Initial guess:
    the Thomas-Fermi profile plus 1e-2 seeded noise.  Step dtau (trap units).
    """
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.choice(grids))
        wp = float(rng.uniform(0.05, 0.2))
        lam = float(rng.uniform(0.5, 4.0))
        g = float(10 ** rng.uniform(0.0, 3.0))
        Om = float(rng.uniform(0.0, 0.7 * wp))
        w = (wp, wp, lam * wp)
        # dx_perp / xi = 2.6 R_perp / n * sqrt(2 mu) = 5.2 mu / (w_perp n)
        mu = res * wp * n / 5.2 * float(rng.uniform(0.6, 1.0))
        R = [math.sqrt(2 * mu) / wa for wa in w]
        box = tuple(2.6 * r for r in R)
        prob = TrapProblem(n=(n, n, n), box=box, omega=w, g=g, mu=mu, dt=dtau, Omega=Om, precision=precision)
        a = prob.a
        init = dict(name="tf_noise", amp=1.0, r_tf2=[(a / r) ** 2 for r in R], noise_amp=1e-2,
                    seed=int(seed * 1000003 + i), g=g, Omega=Om, omega=w, N=tf_norm(w, g, mu))
        out.append((prob, init))
    return out
