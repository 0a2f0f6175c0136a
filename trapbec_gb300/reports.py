"""Precision reports of the GPU path (no oracle involved).

fp32_vs_fp64(): the 256^3 vortex-ring real-time run (TF background x ring of
radius 8 in z = 0 with 1e-3 phase noise, anisotropic trap (0.05, 0.05, 0.1),
g = 1, dt = 0.005) advanced in complex FP64 and in complex FP32 from the same
initial state; reports the FP32 norm and energy drift relative to the FP64
run and the relative L2 error of psi against it, plus the GB/s of both.
"""
from __future__ import annotations

import time

import numpy as np

from . import abi, units
from .solver import Solver


def _run(prec, n, steps, chunk, psi0=None, seed=1234, form=abi.RK3_THREE_STAGE):
    prob, init = units.vortex_ring_256(prec, n=n, seed=seed)
    s = Solver(prob.to_params())
    s.set_stage_form(form)
    if psi0 is None:
        s.init_state(init["name"], seed=init["seed"], amp=init["amp"], r_tf2=init["r_tf2"],
                     ring_radius=init["ring_radius"], noise_amp=init["noise_amp"])
    else:
        s.set_psi(psi0)
    s.autotune(steps=3)   # tile shape and work order for this grid and form (state restored)
    d0 = s.diag()
    ms = 0.0
    done = 0
    checkpoints = []
    while done < steps:
        k = min(chunk, steps - done)
        s.step_rt(k)
        ms += s.last_kernel_ms()
        done += k
        checkpoints.append((done, s.diag()))
    psi = s.get_psi()
    s.close()
    return prob, d0, checkpoints, psi, ms


def fp32_vs_fp64(n: int = 256, steps: int = 2000, chunk: int = 250, seed: int = 1234) -> dict:
    t0 = time.time()
    prob, d0, ck64, psi64, ms64 = _run(abi.FP64, n, steps, chunk, seed=seed)
    # the FP32 run starts from the FP64 initial state rounded to FP32
    prob64, init = units.vortex_ring_256(abi.FP64, n=n, seed=seed)
    s = Solver(prob64.to_params())
    s.init_state(init["name"], seed=init["seed"], amp=init["amp"], r_tf2=init["r_tf2"],
                 ring_radius=init["ring_radius"], noise_amp=init["noise_amp"])
    psi0 = s.get_psi().astype(np.complex64)
    s.close()
    _, d032, ck32, psi32, ms32 = _run(abi.FP32, n, steps, chunk, psi0=psi0, seed=seed)
    l2 = float(np.linalg.norm(psi32.astype(np.complex128) - psi64) / np.linalg.norm(psi64))
    # the same FP32 run in the psi-difference form (no w array; 64 instead of 80 bytes moved)
    _, d0p, ckp, psip, msp = _run(abi.FP32, n, steps, chunk, psi0=psi0, seed=seed, form=abi.RK3_PSI_DIFF)
    l2p = float(np.linalg.norm(psip.astype(np.complex128) - psi64) / np.linalg.norm(psi64))
    cells = n ** 3
    out = {
        "grid": n, "steps": steps,
        "fp64": {"ms_per_step": ms64 / steps, "gbs_alg": cells * steps * 160 / (ms64 * 1e-3) / 1e9,
                 "norm_drift": ck64[-1][1]["norm"] / d0["norm"] - 1.0,
                 "energy_drift": ck64[-1][1]["energy"] / d0["energy"] - 1.0},
        "fp32": {"ms_per_step": ms32 / steps, "gbs_alg": cells * steps * 80 / (ms32 * 1e-3) / 1e9,
                 "norm_drift": ck32[-1][1]["norm"] / d032["norm"] - 1.0,
                 "energy_drift": ck32[-1][1]["energy"] / d032["energy"] - 1.0},
        "fp32_vs_fp64": {
            "l2_rel_psi": l2,
            "norm_rel": ck32[-1][1]["norm"] / ck64[-1][1]["norm"] - 1.0,
            "energy_rel": ck32[-1][1]["energy"] / ck64[-1][1]["energy"] - 1.0,
            "checkpoints": [{"step": a[0], "norm_rel": b[1]["norm"] / a[1]["norm"] - 1.0,
                             "energy_rel": b[1]["energy"] / a[1]["energy"] - 1.0}
                            for a, b in zip(ck64, ck32)],
        },
        "fp32_psi_diff": {"ms_per_step": msp / steps, "gbs_alg": cells * steps * 80 / (msp * 1e-3) / 1e9,
                          "norm_drift": ckp[-1][1]["norm"] / d0p["norm"] - 1.0,
                          "energy_drift": ckp[-1][1]["energy"] / d0p["energy"] - 1.0,
                          "vs_fp64": {"l2_rel_psi": l2p, "norm_rel": ckp[-1][1]["norm"] / ck64[-1][1]["norm"] - 1.0,
                                      "energy_rel": ckp[-1][1]["energy"] / ck64[-1][1]["energy"] - 1.0}},
        "wall_s": time.time() - t0,
        "energy_trap_units_fp64": prob.energy_to_trap(ck64[-1][1]["energy"]),
    }
    return out


def imag_step_bound(prob: units.TrapProblem) -> float:
    """Trap-units imaginary step at the RK3 stability bound of the
    discretised operator: the imaginary-time stage applies 1/2 dtau' rhs with
    rhs = lap psi + (1 - |psi|^2 - pot) psi, whose largest magnitude is at
    most (1088/180) sum 1/h'^2 (the 6th-order Laplacian at the grid's
    Nyquist mode) + max pot (the box corner: sum harm_w / 4) + max |psi|^2
    (~1); RK3 is stable on [-2.51, 0]; dtau = dtau' / (2 mu)."""
    p = prob.to_params()
    lam = (1088.0 / 180.0) * sum((m / L) ** 2 for m, L in ((p.nx, p.lx), (p.ny, p.ly), (p.nz, p.lz)))
    lam += (p.harm_wx + p.harm_wy + p.harm_wz) / 4.0 + 1.0
    return 2.0 * 2.51 / lam / (2.0 * prob.mu)


def quench_ground_state(n: int = 512, seed: int = 99, frac: float = 0.7, tol: float = 1e-8,
                        max_steps: int = 6000):
    """The quench's starting state: the Thomas-Fermi + 1e-2 noise cloud of the
    512^3 rotating trap relaxed in imaginary time (FP32 state, FP64
    renormalisation and energy test: RK3_RENORM) at Omega = 0, the rotation at
    the start of the ramp, until |dE|/|E| <= tol or max_steps, with the
    imaginary step at `frac` of imag_step_bound (0.0117 trap units at 512^3
    on [-64, 64]^3).  Returns (psi complex64, steps taken, last |dE|/|E|,
    device ms, dtau, the state's chemical potential in reference units)."""
    prob, init = units.rotating_quench_512(abi.FP32, n=n, seed=seed)
    dtau = frac * imag_step_bound(prob)
    p = prob.to_params()
    s = Solver(p)
    s.init_state(init["name"], seed=init["seed"], amp=init["amp"], r_tf2=init["r_tf2"],
                 noise_amp=init["noise_amp"])
    s.set_scalar(abi.SCALAR_DT_RE, 2.0 * prob.mu * dtau)
    steps, dE = s.step_imag(max_steps, abi.IMAG_RK3_RENORM, tol)
    ms = s.last_kernel_ms()
    mu = s.diag()["mu"]
    psi = s.get_psi()
    s.close()
    return psi, steps, dE, ms, dtau, mu


def quench_checkpoints(n: int = 512, steps: int = 1000, every: int = 500, chunk: int = 50,
                       ramp_steps: int = 5000, fp32_steps: int = 5000, seed: int = 99,
                       relax_tol: float = 1e-8, relax_max_steps: int = 6000, gauge: str = "state_mu",
                       ground=None) -> dict:
    """The 512^3 rotating quench (omega_perp = 0.02, omega_z = 0.04, g = 1,
    dt = 0.004, Omega ramped 0 -> 0.8 omega_perp over `ramp_steps`) from the
    imaginary-time ground state of `quench_ground_state`, advanced in complex
    FP32 for `fp32_steps` (the whole ramp) and in complex FP64 for the first
    `steps`; norm and energy at every `every` steps, FP32 relative to FP64
    where both ran, the FP32 run's own drift over the whole ramp, and the L2
    error of psi at step `steps`.

    `gauge` picks the unit scale mu of the reference units (the equation's
    chemical potential, which is 1 in those units):
      "tf_mu"    -- the Thomas-Fermi estimate the cloud was built with;
      "state_mu" -- the relaxed state's own chemical potential.
    The physics is the same (trap units), but in the "tf_mu" units the ground
    state turns its phase by dt' (mu_state - mu) / 2 per step, and in FP32
    the real part's second-order decrease under that slow rotation is below
    half an ulp in most cells: round-to-nearest keeps the old value, and |psi|
    grows by the square of the phase turned until the per-step change
    reaches an ulp.  In the state's own units the ground state is
    stationary and that bias is gone.  `ground` reuses a
    quench_ground_state() result."""
    import math
    t0 = time.time()
    if ground is None:
        ground = quench_ground_state(n, seed, tol=relax_tol, max_steps=relax_max_steps)
    psi0, rsteps, rdE, rms, rdtau, mu_ref = ground
    prob0, _ = units.rotating_quench_512(abi.FP32, n=n, seed=seed)
    if gauge == "tf_mu":
        mu_unit = prob0.mu
    elif gauge == "state_mu":
        mu_unit = prob0.mu_to_trap(mu_ref)
    else:
        raise ValueError(f"unknown gauge {gauge!r}")
    start32 = (psi0.astype(np.complex128) * math.sqrt(prob0.mu / mu_unit)).astype(np.complex64)
    runs = {}
    for prec, nsteps in ((abi.FP64, steps), (abi.FP32, max(steps, fp32_steps))):
        prob, init = units.rotating_quench_512(prec, n=n, seed=seed)
        prob.mu = mu_unit
        s = Solver(prob.to_params())
        s.set_psi(start32 if prec == abi.FP32 else start32.astype(np.complex128))
        d0 = s.diag()
        ck = []
        ms = 0.0
        done = 0
        psi_at = None
        while done < nsteps:
            k = min(chunk, nsteps - done)
            s.set_scalar(abi.SCALAR_OMEGA_Z, prob.omega_z_for(init["omega_final"] * min(1.0, done / ramp_steps)))
            s.step_rt(k)
            ms += s.last_kernel_ms()
            done += k
            if done % every == 0:
                ck.append((done, s.diag()))
            if done == steps:
                psi_at = s.get_psi()
        runs[prec] = (d0, ck, psi_at, ms, nsteps)
        s.close()
    d64, ck64, psi64, ms64, n64 = runs[abi.FP64]
    d32, ck32, psi32, ms32, n32 = runs[abi.FP32]
    l2 = float(np.linalg.norm((psi32.astype(np.complex128) - psi64).ravel()) / np.linalg.norm(psi64.ravel()))
    ck32_at = {a: b for a, b in ck32}
    return {
        "grid": n, "steps_fp64": n64, "steps_fp32": n32,
        "start": {"state": "imaginary-time ground state at Omega = 0 (FP32, RK3_RENORM) of the TF + 1e-2 noise cloud",
                  "relax_steps": rsteps, "relax_dtau_trap_units": rdtau, "relax_rel_dE": rdE, "relax_tol": relax_tol,
                  "relax_ms_device": rms, "mu_state_trap_units": prob0.mu_to_trap(mu_ref)},
        "gauge": gauge, "mu_unit_trap_units": mu_unit,
        "omega_ramp": f"0 -> 0.8 omega_perp over {ramp_steps} steps, per {chunk}-step chunk",
        "fp64": {"ms_per_step": ms64 / n64, "norm_drift": ck64[-1][1]["norm"] / d64["norm"] - 1.0,
                 "energy_drift": ck64[-1][1]["energy"] / d64["energy"] - 1.0},
        "fp32": {"ms_per_step": ms32 / n32, "norm_drift": ck32[-1][1]["norm"] / d32["norm"] - 1.0,
                 "energy_drift": ck32[-1][1]["energy"] / d32["energy"] - 1.0,
                 "checkpoints": [{"step": a, "norm_drift": b["norm"] / d32["norm"] - 1.0,
                                  "energy_drift": b["energy"] / d32["energy"] - 1.0} for a, b in ck32]},
        "fp32_vs_fp64": {
            "l2_rel_psi_at": steps, "l2_rel_psi": l2,
            # the same starting values evaluated by each precision's diagnostics
            "start": {"norm_rel": d32["norm"] / d64["norm"] - 1.0, "energy_rel": d32["energy"] / d64["energy"] - 1.0},
            "checkpoints": [{"step": a, "norm_rel": ck32_at[a]["norm"] / b["norm"] - 1.0,
                             "energy_rel": ck32_at[a]["energy"] / b["energy"] - 1.0}
                            for a, b in ck64],
        },
        "wall_s": time.time() - t0,
    }


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="FP32 against FP64 precision reports on the GPU")
    ap.add_argument("which", choices=["ring256", "quench512"])
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--steps", type=int, default=None)
    a = ap.parse_args()
    if a.which == "ring256":
        r = fp32_vs_fp64(n=a.n or 256, steps=a.steps or 2000)
    else:
        n = a.n or 512
        ground = quench_ground_state(n)
        r = {g: quench_checkpoints(n=n, steps=a.steps or 1000, gauge=g, ground=ground)
             for g in ("state_mu", "tf_mu")}
    print(json.dumps(r, indent=1))
