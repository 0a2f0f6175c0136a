"""Shared helpers of the tests (problem set-ups in the reference's units)."""
import numpy as np

from trapbec_gb300 import abi
from trapbec_gb300.abi import Params, default_params


def params(n=(16, 16, 16), L=(8.0, 8.0, 8.0), prec=abi.FP64, bc=abi.BC_ZERO, pot="zero",
           dt=0.005, omega=0.0, vx=0.0, harm=(0.0, 0.0, 0.0), periodicz=0, two_dim=0,
           nproc=(1, 1), gamma=0.0, lbeam=0) -> Params:
    p = default_params()
    p.nx, p.ny, p.nz = n
    p.lx, p.ly, p.lz = L
    p.precision = prec
    p.boundaries = bc
    p.potential = abi.POTENTIALS[pot]
    p.dt_re, p.dt_im = dt, 0.0
    p.omega_z = omega
    p.advective_vx = vx
    p.harm_wx, p.harm_wy, p.harm_wz = harm
    p.periodicz = periodicz
    p.two_dim = two_dim
    p.nprocx, p.nprocy = nproc
    p.gamma = gamma
    p.lbeam = lbeam
    return p


def coords(p: Params):
    """Cell-centred coordinates of a single-rank run (initial.f90:34-42)."""
    xs = []
    for n, L in ((p.nx, p.lx), (p.ny, p.ly), (p.nz, p.lz)):
        i = np.arange(1, n + 1)
        xs.append((2 * i - 1) / (2.0 * n) * L - L / 2.0)
    return xs


def smooth_state(p: Params, seed=0, amp=1.0):
    """A smooth complex test state: Gaussian envelope x random low modes."""
    rng = np.random.default_rng(seed)
    x, y, z = coords(p)
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    env = np.exp(-(X ** 2 / (0.08 * p.lx ** 2) + Y ** 2 / (0.08 * p.ly ** 2) + Z ** 2 / (0.08 * p.lz ** 2)))
    ph = np.zeros_like(X)
    for _ in range(3):
        k = rng.integers(-2, 3, size=3) * 2 * np.pi / np.array([p.lx, p.ly, p.lz])
        ph += rng.uniform(-1, 1) * np.sin(k[0] * X + k[1] * Y + k[2] * Z + rng.uniform(0, 6))
    return (amp * env * np.exp(1j * ph)).astype(np.complex128)


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
