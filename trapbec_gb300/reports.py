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


def _run(prec, n, steps, chunk, psi0=None, seed=1234):
    prob, init = units.vortex_ring_256(prec, n=n, seed=seed)
    s = Solver(prob.to_params())
    if psi0 is None:
        s.init_state(init["name"], seed=init["seed"], amp=init["amp"], r_tf2=init["r_tf2"],
                     ring_radius=init["ring_radius"], noise_amp=init["noise_amp"])
    else:
        s.set_psi(psi0)
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
        "wall_s": time.time() - t0,
        "energy_trap_units_fp64": prob.energy_to_trap(ck64[-1][1]["energy"]),
    }
    return out


def quench_checkpoints(n: int = 512, steps: int = 1000, every: int = 500, chunk: int = 50,
                       ramp_steps: int = 5000, seed: int = 99) -> dict:
    """The 512^3 rotating quench (omega_perp = 0.02, omega_z = 0.04, g = 1,
    dt = 0.004, Omega ramped 0 -> 0.8 omega_perp over `ramp_steps`) advanced
    in complex FP32 and in complex FP64 from the same initial state; norm and
    energy at every `every` steps, FP32 relative to FP64, and the L2 error
    of psi at the end."""
    t0 = time.time()
    runs = {}
    psi0 = None
    for prec in (abi.FP64, abi.FP32):
        prob, init = units.rotating_quench_512(prec, n=n, seed=seed)
        s = Solver(prob.to_params())
        if psi0 is None:
            s.init_state(init["name"], seed=init["seed"], amp=init["amp"], r_tf2=init["r_tf2"],
                         noise_amp=init["noise_amp"])
            psi0 = s.get_psi()
        else:
            s.set_psi(psi0.astype(np.complex64))
        d0 = s.diag()
        ck = []
        ms = 0.0
        done = 0
        while done < steps:
            k = min(chunk, steps - done)
            s.set_scalar(abi.SCALAR_OMEGA_Z, prob.omega_z_for(init["omega_final"] * min(1.0, done / ramp_steps)))
            s.step_rt(k)
            ms += s.last_kernel_ms()
            done += k
            if done % every == 0:
                ck.append((done, s.diag()))
        runs[prec] = (d0, ck, s.get_psi(), ms)
        s.close()
    d64, ck64, psi64, ms64 = runs[abi.FP64]
    d32, ck32, psi32, ms32 = runs[abi.FP32]
    l2 = float(np.linalg.norm((psi32.astype(np.complex128) - psi64).ravel()) / np.linalg.norm(psi64.ravel()))
    return {
        "grid": n, "steps": steps, "omega_ramp": f"0 -> 0.8 omega_perp over {ramp_steps} steps, per {chunk}-step chunk",
        "fp64": {"ms_per_step": ms64 / steps, "norm_drift": ck64[-1][1]["norm"] / d64["norm"] - 1.0,
                 "energy_drift": ck64[-1][1]["energy"] / d64["energy"] - 1.0},
        "fp32": {"ms_per_step": ms32 / steps, "norm_drift": ck32[-1][1]["norm"] / d32["norm"] - 1.0,
                 "energy_drift": ck32[-1][1]["energy"] / d32["energy"] - 1.0},
        "fp32_vs_fp64": {
            "l2_rel_psi": l2,
            "checkpoints": [{"step": a[0], "norm_rel": b[1]["norm"] / a[1]["norm"] - 1.0,
                             "energy_rel": b[1]["energy"] / a[1]["energy"] - 1.0}
                            for a, b in zip(ck64, ck32)],
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
        r = quench_checkpoints(n=a.n or 512, steps=a.steps or 1000)
    print(json.dumps(r, indent=1))
