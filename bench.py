"""Benchmark of the TrapBEC hot path on GB300.

Workload (default): the rotating-trap quench at 512^3 in complex FP32 with
FP64 diagnostics, on [-64,64]^3, omega_perp = 0.02, omega_z = 0.04, g = 1,
dt = 0.004, Omega ramped linearly towards 0.8 omega_perp.  One bench step is
one full low-storage RK3 step (three fused stage kernels) over the whole
grid.  The metric is grid-point updates per second (one grid point advanced
by one RK3 step).  The run starts from the ground state of the trap at
Omega = 0: the seeded Thomas-Fermi cloud with 1e-2 noise relaxed in
imaginary time on the GPU (FP32 state, FP64 renormalisation and energy).
Each array is 1 GiB, far larger than the 129 MB L2, so no flush is needed
between steps.

Beside the timed FP32 run the line carries: the same start advanced in FP64
and in the compensated FP32 form over a fixed number of steps, with each FP32
form's norm, energy and L2 error against FP64 (fp32_vs_fp64); the end-to-end
rate through the C ABI with host buffers; the CPU restatement's rate on the
host cores; the batched imaginary-time ground states (64 instances) and the
surrogate-against-Thomas-Fermi warm start.

Output: one JSON line (see the keys below); `--impl reference` times the CPU
restatement of the reference's algorithm on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "grid-pt updates/s at 512^3 FP32 vs FP64 (HBM %); imag-time wall to dE<1e-10: NN vs TF"
UNIT = "grid-point updates/s"
# HBM bytes per grid point and RK3 step each real-time form moves (complex
# FP32; FP64 doubles them): three stages S1 24 + S2 32 + S3 24; the deferred
# form stores no psi1 (S1 16); the compensated state reads and rewrites its
# remainder in every stage (+48); the psi-difference form stores no w
# (S1 16 + S2 24 + S3 24).
FORM_BYTES = {0: 80.0, 1: 72.0, 2: 128.0, 3: 64.0}
# Algorithmic bytes of the roofline: the three-stage 2N-storage schedule of
# the state a form carries (psi: 80 B; psi and its remainder: 128 B).  A form
# that moves fewer bytes for the same state keeps this figure, so its
# fraction can exceed that of the unfused schedule; its own bytes are
# reported beside it.
ALG_BYTES = {0: 80.0, 1: 80.0, 2: 128.0, 3: 80.0}
FORM_PROFILE = {1: "deferred", 2: "compensated", 3: "psi_diff"}
FORM_TEXT = {0: "three full stages",
             1: "deferred psi1: stage 1 stores w1 only, stage 2 forms psi1 = psi0 + w1/3 (bit-identical)",
             2: "compensated state (remainder array, difference-form stencil)",
             3: ("psi difference: no w array; stage 1 stores psi1 only, stages 2 and 3 recover the previous "
                 "stage's w as (psi_k - psi_(k-1)) / B_(k-1) from the two psi arrays")}


def load_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_bf16_peak():
    """Dense BF16 TFLOP/s of this GPU as a burst (cuBLAS, measured), else the fallback figure."""
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        if "bf16_tflops" in d:
            return float(d["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


def surrogate_kernels():
    """Tensor-core rate of the surrogate's convolutions at 128^3, batch 2:
    one forward pass and one training step (forward, input and weight
    gradients, clipping, Adam), device time from events, against the
    measured BF16 burst peak."""
    from trapbec_gb300 import surrogate
    r = surrogate.time_passes(128, 2, 5)
    peak, kind = load_bf16_peak()
    return {"grid": 128, "batch": 2, "forward_ms": r["forward_ms"], "train_step_ms": r["train_step_ms"],
            "conv_gflop_forward": r["conv_gflop_forward"], "conv_gflop_backward": r["conv_gflop_backward"],
            "forward": {"bound": "tensor", "achieved": r["conv_tflops_forward"], "peak": peak, "unit": "TFLOP/s",
                        "frac": r["conv_tflops_forward"] / peak, "peak_kind": kind},
            "train_step": {"bound": "tensor", "achieved": r["conv_tflops_train_step"], "peak": peak,
                           "unit": "TFLOP/s", "frac": r["conv_tflops_train_step"] / peak, "peak_kind": kind},
            "kernels": "tcgen05: conv3_tc_kernel (16/32 channels), conv3_tcs_kernel (64/128, streamed weights), "
                       "conv3_wgrad_tc_kernel (weight gradients)"}


def profile_traffic(prec_tag: str, tz: int | None = None, ty: int | None = None, form: str = ""):
    """DRAM bytes per grid point per stage launch from the committed ncu summary
    of the full-size launch list of the tile shape and RK3 form that ran
    (profiles/stage_tiled_<prec>_512_<tz>x<ty>[_<form>].txt; the 128 x 8 FP32
    three-stage default is profiles/stage_tiled_fp32_512.txt)."""
    if tz is None and ty is None:
        tz, ty = 128, 8
    sfx = f"_{form}" if form else ""
    path = os.path.join(HERE, "profiles", f"stage_tiled_{prec_tag}_512_{tz}x{ty}{sfx}.txt")
    if form:
        if not os.path.exists(path):
            return None
        m = re.search(r"dram_bytes_per_point_per_launch:\s*([0-9.eE+-]+)", open(path).read())
        return float(m.group(1)) if m else None
    if not os.path.exists(path):
        if (prec_tag, tz, ty) not in (("fp32", 128, 8), ("fp32", None, None)):
            return None
        path = os.path.join(HERE, "profiles", f"stage_tiled_{prec_tag}_512.txt")
    if not os.path.exists(path):
        return None
    m = re.search(r"dram_bytes_per_point_per_launch:\s*([0-9.eE+-]+)", open(path).read())
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", f"trapbec_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            # let nvidia-smi finish starting (its driver initialisation stalls this
            # process's launches) before the timed region begins: wait for a sample
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                if os.path.getsize(self.path) > 0:
                    break
                time.sleep(0.02)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):  # noqa: D401
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names[1:], f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_problem(n: int, prec):
    from trapbec_gb300 import abi, units
    prob, init = units.rotating_quench_512(prec, n=n)
    return prob, init


def fp64_fma_peak():
    """FP64 FMA instructions per second of the GPU (libtrapbec's peak kernel: long
    independent FMA chains on every SM, CUDA events)."""
    import ctypes as C
    from trapbec_gb300 import abi
    v = C.c_double(0)
    abi.check(abi.load().trapbec_fp64_fma_rate(C.byref(v)), "trapbec_fp64_fma_rate")
    return v.value


# FP64 pipe instructions (DADD, DMUL, DFMA) per grid point of the three stage
# kernels' plain variant with the rotating frame (kernels_tiled.cuh, counted
# per complex operation: add/sub/mul/fma of a pair = 2): Laplacian 38, the two
# first derivatives 20, the frame term 6, potential sum 2, |psi|^2 2, the
# nonlinear rhs 6, the complex multiplier 4, the w update 0/2/2 and the psi
# update 2 -> 80 + 82 + 82.
FP64_OPS_PER_POINT_STEP = 244


def cpu_reference(n: int, steps: int, threads: int | None):
    """Time the oracle (CPU restatement of the reference) on the host cores."""
    from oracle.pyoracle import Oracle
    from trapbec_gb300 import abi
    from trapbec_gb300.abi import InitArgs
    prob, init = make_problem(n, abi.FP32)
    p = prob.to_params()
    p.omega_z = prob.omega_z_for(0.4 * init["omega_final"])
    if threads:
        Oracle.set_threads(threads)
    cores = Oracle.max_threads()
    o = Oracle(p)
    a = InitArgs()
    a.seed = init["seed"]; a.amp = init["amp"]; a.noise_amp = init["noise_amp"]
    for i in range(3):
        a.r_tf2[i] = init["r_tf2"][i]
    o.init_state(init["name"], a)
    o.step_rt(1)  # warm caches and pages
    t0 = time.perf_counter()
    o.step_rt(steps)
    dt = time.perf_counter() - t0
    return n ** 3 * steps / dt, cores, dt


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.n
    # a bounded sample of the workload: the full 512^3 grid, a few steps
    # (about 10 s on 16 host cores), repeated for each timed bench step
    k = max(1, min(args.steps, args.cpu_steps))
    val, cores, dt = cpu_reference(n, k, None)
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
        "steps": k, "warmup": 1, "ms_per_step": 1e3 * dt / k, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 (f32)", "data": "synthetic",
        "config": {"workload": f"rotating-trap RK3 quench {n}^3 complex FP32", "grid": [n, n, n],
                   "l2_flush": "inputs larger than L2 (1 GiB per array)"},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{k} RK3 step(s) of the full {n}^3 grid (OpenMP over x)"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference (Fortran 90 + MPI) has no Fortran compiler or MPI on this image; "
                "its algorithm is timed through the CPU restatement (oracle/)",
    }
    print(json.dumps(line), flush=True)


def timed_steps(s, steps, chunk, omega_of_step, start_step=0):
    """Run `steps` RK3 steps in chunks (Omega updated per chunk); returns
    (device ms of the stage kernels, launches)."""
    from trapbec_gb300 import abi
    ms = 0.0
    l0 = s.launch_count()
    done = 0
    while done < steps:
        k = min(chunk, steps - done)
        s.set_scalar(abi.SCALAR_OMEGA_Z, omega_of_step(start_step + done))
        s.step_rt(k)
        ms += s.last_kernel_ms()
        done += k
    return ms, s.launch_count() - l0


def imag_leg(args):
    """Batched imaginary-time ground states from the Thomas-Fermi guess (the
    64-instance workload): device time (events around the whole
    graph-replayed loop) until every instance meets the stop test or
    max_steps.  The stop test is the workload's |dE| < tol on the energy per
    particle in trap units (the wave function normalised to one, as the
    Thomas-Fermi-scaled interaction g implies): |E_n - E_{n-1}| / N * 2 mu <
    tol, formed in FP64 on the device."""
    from trapbec_gb300 import abi, units
    from trapbec_gb300.batch import BatchSolver
    draws = units.ground_state_draws(args.imag_count, args.imag_seed, grids=tuple(args.imag_grids),
                                     precision=abi.FP32)
    b = BatchSolver([p.to_params() for p, _ in draws])
    for i, (p, ini) in enumerate(draws):
        b.init_state(i, ini["name"], seed=ini["seed"], amp=ini["amp"], r_tf2=ini["r_tf2"],
                     noise_amp=ini["noise_amp"])
    b.set_imag_stop(abi.STOP_ABS_PER_NORM, [p.mu_to_trap(1.0) for p, _ in draws])
    t0 = time.perf_counter()
    out = b.solve(max_steps=args.imag_max_steps, tol=args.imag_tol, check_every=200)
    wall = time.perf_counter() - t0
    st = b.stats()
    stat = [b.status(i) for i in range(len(draws))]
    conv = [x["converged"] > 0 for x in stat]
    cells = sum(p.n[0] * p.n[1] * p.n[2] for p, _ in draws)
    b.close()
    fast = [d["Omega"] / d["omega"][0] > 0.5 for _, d in draws]
    return {"guess": "thomas_fermi+1e-2 noise", "instances": len(draws), "cells": cells,
            "grids": sorted(set(p.n[0] for p, _ in draws)),
            "stop": "|d(E/N)| < tol, energy per particle in trap units (FP64)", "tol": args.imag_tol,
            "dtau_trap_units": 0.002, "max_steps": args.imag_max_steps,
            "converged": int(sum(conv)), "steps_median": float(statistics.median(out["steps"])),
            "steps_max": int(max(out["steps"])), "solve_ms_device": st["solve_ms"], "wall_s": wall,
            "not_converged_fast_rotating": int(sum(1 for c, f in zip(conv, fast) if not c and f)),
            "not_converged_slow_rotating": int(sum(1 for c, f in zip(conv, fast) if not c and not f)),
            "last_dE_per_particle_not_converged": [x["rel"] for x in stat if x["converged"] <= 0],
            "tile": [st["tile_z"], st["tile_y"]],
            "precision": ("c64 state; norm and energy sums compensated float-float (FP32 arithmetic, ~44 bits) "
                          "with the kinetic term in difference form; renormalisation, energy and stop test in FP64")}


def ring_leg(args, peak):
    """The 256^3 vortex-ring workload (TF background x a ring of radius 8 in
    z = 0 with 1e-3 seeded phase noise, trap (0.05, 0.05, 0.1), g = 1,
    dt = 0.005): 2000 RK3 steps in complex FP64 and in complex FP32 from the
    same start; GB/s on algorithmic bytes, HBM fraction, and the FP32 run's
    norm/energy drift and L2 error against the FP64 run."""
    from trapbec_gb300 import reports
    r = reports.fp32_vs_fp64(n=256, steps=args.ring_steps, chunk=250)
    for k in ("fp32", "fp64", "fp32_psi_diff"):
        r[k]["hbm_frac"] = r[k]["gbs_alg"] / peak
    r["workload"] = "vortex ring 256^3, FP64 and FP32 from the same start"
    return r


def stretch_leg(args, peak):
    """The quench workload's 1024^3 stretch size in complex FP32 (25.8 GB of
    state): the headline's form on the autotuned tile, `stretch_steps` RK3
    steps at the mid-ramp rotation from the seeded TF cloud (no ground state:
    its relaxation at this size would dominate the run), device time."""
    from trapbec_gb300 import Solver, abi
    n = 1024
    prob, init = make_problem(n, abi.FP32)
    s = Solver(prob.to_params())
    s.set_stage_form(args.stage_form)
    tune = None if args.no_autotune else s.autotune(steps=3)
    s.init_state(init["name"], seed=init["seed"], amp=init["amp"], r_tf2=init["r_tf2"], noise_amp=init["noise_amp"])
    s.set_scalar(abi.SCALAR_OMEGA_Z, prob.omega_z_for(0.5 * init["omega_final"]))
    s.step_rt(3)
    steps = args.stretch_steps
    s.step_rt(steps)
    ms = s.last_kernel_ms()
    form = s.stage_form()
    tz, ty = s.tile_shape(real_time=True)
    s.close()
    cells = n ** 3
    ach = cells * steps * ALG_BYTES[form] / (ms * 1e-3) / 1e9
    return {"grid": [n, n, n], "steps": steps, "ms_per_step": ms / steps, "value": cells * steps / (ms * 1e-3),
            "unit": UNIT, "tile": [tz, ty], "autotune": tune, "rk3_form": FORM_TEXT[form],
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "algorithmic_bytes_per_point_step": ALG_BYTES[form],
                         "form_bytes_per_point_step": FORM_BYTES[form],
                         "frac_of_form_bytes": cells * steps * FORM_BYTES[form] / (ms * 1e-3) / 1e9 / peak}}


def warmstart_leg(args):
    """Imaginary-time relaxation to |d(E/N)| < tol at 128^3 from the
    surrogate's guess against the Thomas-Fermi + 1e-2 noise guess, on the
    first draws held out from the surrogate's training set (the committed
    weights were trained on draws 0..TRAIN_DRAWS-1 of seed TRAIN_SEED).
    Both relaxations run batched; device time from events around each solve."""
    from trapbec_gb300 import abi, units, surrogate
    n0 = surrogate.TRAIN_DRAWS
    draws = units.ground_state_draws(n0 + args.ws_count, surrogate.TRAIN_SEED, grids=(128,),
                                     precision=abi.FP32)[n0:]
    net = surrogate.Surrogate(128, 2, seed=0)
    net.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "trapbec_gb300", "weights",
                          "surrogate_128.npz"))
    r = surrogate.compare(net, draws, tol=args.imag_tol, max_steps=args.ws_max_steps, stop="per_particle",
                          subset_rerun=True)
    med = lambda v: float(statistics.median(v))
    return {
        "grid": 128, "instances": len(draws), "held_out": f"draws {n0}..{n0 + len(draws) - 1} of seed {surrogate.TRAIN_SEED}",
        "stop": "|d(E/N)| < tol, energy per particle in trap units (FP64)", "tol": args.imag_tol,
        "dtau_trap_units": 0.002, "max_steps": args.ws_max_steps,
        "surrogate_params": net.np, "nn_used": r["nn_used"],
        "steps_tf": r["tf"]["steps"], "steps_nn": r["nn"]["steps"],
        "converged_tf": int(sum(r["tf"]["converged"])), "converged_nn": int(sum(r["nn"]["converged"])),
        "steps_ratio_median": r["steps_ratio_median"], "steps_ratio_median_nn_used": r["steps_ratio_median_nn_used"],
        "steps_ratio_total_both_converged": r["steps_ratio_total_both_converged"],
        "device_ms_tf": r["tf"]["solve_ms_device"], "device_ms_nn": r["nn"]["solve_ms_device"],
        "nn_inference_ms": r["nn_inference_ms"], "selection_ms_device": r["selection_ms_device"],
        "wall_ratio_device": r["wall_ratio_device"],
        "wall_ratio_note": "TF solve / (NN-arm solve + inference + the selector's energy evaluations), device times",
        "final_energy_rel_diff_max": r["final_energy_rel_diff_max"],
        "same_end_state": r["same_end_state"],
        "guess_rmse_median_tf": med(r["guess_rmse_tf"]), "guess_rmse_median_nn": med(r["guess_rmse_nn"]),
        "fallback": "TF guess where its energy at the same norm is lower, and for Omega/omega_perp > 0.5 "
                    "(bistable: vortex nucleation from the TF guess)",
        "tf_kept_fast_rotation": r["tf_kept_fast_rotation"],
        # the draws whose plain (TF-guess) relaxation reaches the tolerance, relaxed again in both arms
        # as batches of their own: the batch wall-time ratio of the set the plain method solves, not
        # set by the fast-rotating draws that run max_steps in both arms
        "tf_converged_set": r["subset_tf_converged"],
    }


def max_over_ranks(values, dist, device):
    """Each of `values` replaced by its maximum over the ranks (the slowest rank's
    times); unchanged on a single process."""
    if dist is None:
        return list(values)
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def aggregate_ranks(ms_local, units_local, dist, device):
    """Whole-job figure of N replica ranks: the slowest rank's timed milliseconds
    (max over ranks) and the units all ranks processed in that time."""
    import torch
    t = torch.tensor([ms_local, float(units_local)], dtype=torch.float64, device=device)
    if dist is not None:
        mx = t[:1].clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        tot = t[1:].clone()
        dist.all_reduce(tot, op=dist.ReduceOp.SUM)
        t = torch.cat([mx, tot])
    ms = float(t[0].item())
    return ms, float(t[1].item()) / (ms * 1e-3)


def run_gpu_arm(args):
    import numpy as np
    import torch
    from trapbec_gb300 import Solver, abi

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    n = args.n
    prec = abi.FP64 if args.fp64_only else abi.FP32
    prob, init = make_problem(n, prec)
    p = prob.to_params()
    s = Solver(p)
    if args.kernel:
        s.set_kernel(*args.kernel)
    s.set_stage_form(args.stage_form)
    tune = None
    if args.kernel is None and not args.no_autotune:
        tune = s.autotune(steps=8)   # tile shape and work order for this grid (state restored)
    if args.work_chunk is not None:
        s.set_chunk(args.work_chunk)   # a given work order (negative: the strided order)
    s.init_state(init["name"], seed=init["seed"] + rank, amp=init["amp"], r_tf2=init["r_tf2"],
                 noise_amp=init["noise_amp"])
    ramp_steps = 5000
    om_final = init["omega_final"]

    def omega_of_step(k):
        return prob.omega_z_for(om_final * min(1.0, k / ramp_steps))

    # the start: the ground state at Omega = 0 (imaginary time on the GPU)
    ground = None
    if args.start == "ground":
        from trapbec_gb300 import reports
        ground = reports.quench_ground_state(n, seed=init["seed"] + rank)
        s.set_psi(ground[0])
    chunk = args.chunk
    d0 = s.diag()
    # warm-up (untimed)
    timed_steps(s, args.warmup, chunk, omega_of_step, 0)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ms, launches = timed_steps(s, args.steps, chunk, omega_of_step, args.warmup)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    d1 = s.diag()
    cells = n ** 3
    ms, value = aggregate_ranks(ms, cells * args.steps, dist, "cuda")
    peak, peak_kind = load_peaks()
    # algorithmic bytes per grid point per RK3 step: S1 24 + S2 32 + S3 24 (complex FP32);
    # the deferred form stores no psi1 (S1 16 B); FP64 doubles every figure
    form_run = s.stage_form()
    deferred = form_run == abi.RK3_DEFERRED
    bpc = ALG_BYTES[form_run] * (1.0 if prec == abi.FP32 else 2.0)
    fbc = FORM_BYTES[form_run] * (1.0 if prec == abi.FP32 else 2.0)
    achieved = cells * args.steps * bpc / (ms * 1e-3) / 1e9
    achieved_form = cells * args.steps * fbc / (ms * 1e-3) / 1e9
    tag = "fp32" if prec == abi.FP32 else "fp64"
    tz_run, ty_run = s.tile_shape(real_time=True)
    tpp = profile_traffic(tag, tz_run, ty_run, form=FORM_PROFILE.get(form_run, ""))
    traffic = tpp * cells if tpp else None

    kernel_name = "tiled TMA stage kernel" if args.kernel is None or args.kernel[0] != 1 else "per-cell stage kernel"

    # ---- end to end through the C ABI with pinned host buffers ----------------
    e2e = None
    if not args.no_e2e:
        shots = args.shots
        # both host buffers are allocated pinned (page-locked by the CUDA host allocator) and the
        # tensors that own them are kept for the whole leg
        cdt = torch.complex64 if prec == abi.FP32 else torch.complex128
        host_t = torch.empty(cells, dtype=cdt, pin_memory=True)
        host_out_t = torch.empty(cells, dtype=cdt, pin_memory=True)
        host, host_out = host_t.numpy(), host_out_t.numpy()
        host[:] = s.get_psi().reshape(-1)
        host_out[:] = 0
        reps = max(1, args.e2e_reps)

        parts = []
        serial_diag = []

        def e2e_call(r):
            ta = time.perf_counter()
            s.set_psi(host.reshape(s.shape))                       # H2D of the state (queued on the stream)
            s.set_scalar(abi.SCALAR_OMEGA_Z, omega_of_step(args.warmup + args.steps + r * shots))
            s.step_rt(shots)                                       # RK3 steps (waits for the H2D and the steps)
            tb = time.perf_counter()
            steps_ms = s.last_kernel_ms()
            serial_diag[:] = [s.diag()]                            # FP64 diagnostics (Psi_info/Psi_norm, E)
            tc = time.perf_counter()
            s.get_psi(out=host_out)                                # D2H of the state into pinned memory
            td = time.perf_counter()
            parts.append({"set_psi_and_steps_ms": 1e3 * (tb - ta), "steps_device_ms": steps_ms,
                          "diag_ms": 1e3 * (tc - tb), "get_psi_ms": 1e3 * (td - tc)})

        e2e_call(0)                                                # untimed warm-up call
        parts.clear()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        call_ms = []
        for r in range(reps):
            tc = time.perf_counter()
            e2e_call(r)
            call_ms.append(1e3 * (time.perf_counter() - tc))
        torch.cuda.synchronize()
        et = time.perf_counter() - t0
        serial_last = host_out.copy()

        def e2e_pipelined(nrep):
            """The same calls, queued ahead with the host copies overlapped: call r+1's
            steps are queued behind call r's diagnostics before the host waits for those,
            call r+2's state goes up (set_psi_async) while call r+1's steps run, and call
            r's state comes back (get_psi_async) while call r+1's steps run, so each copy
            has a whole block of steps to hide in.  The caller takes each call's
            diagnostics and state before the next call's are asked for."""
            marks = []

            def queue_steps(r):
                s.set_scalar(abi.SCALAR_OMEGA_Z, omega_of_step(args.warmup + args.steps + r * shots))
                s.step_rt_async(shots)                             # takes call r's queued state

            s.set_psi_async(host)                                  # call 0's state
            queue_steps(0)
            if nrep > 1:
                s.set_psi_async(host)                              # call 1's state, during call 0's steps
            for r in range(nrep):
                s.get_psi_async(host_out)                          # D2H of call r's state, after its steps
                s.diag_async()                                     # FP64 diagnostics of call r's state
                if r + 1 < nrep:
                    queue_steps(r + 1)                             # call r+1's steps, queued behind them
                if r + 2 < nrep:
                    s.set_psi_async(host)                          # H2D of call r+2's state
                diags.append(s.diag_wait())                        # call r's diagnostics on the host
                s.wait_psi()                                       # call r's state on the host
                marks.append(time.perf_counter())
            s.synchronize()
            marks.append(time.perf_counter())
            return marks

        diags = []

        e2e_pipelined(1)                                           # untimed warm-up (allocates the copy buffers)
        host_out[:] = 0
        diags.clear()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        marks = e2e_pipelined(reps)
        torch.cuda.synchronize()
        ep = time.perf_counter() - t0
        et, ep = max_over_ranks([et, ep], dist, "cuda")         # the slowest rank's times for both loops
        pipe_ms = [1e3 * (b - a) for a, b in zip([t0] + marks[:-2], marks[:-1])]
        same = bool(np.array_equal(host_out.view(np.uint8), serial_last.view(np.uint8)) and
                    diags[-1] == serial_diag[-1])
        e2e = {"value": world * cells * shots * reps / ep, "unit": UNIT,
               "h2d_bytes_per_step": int(cells * host.itemsize / shots),
               "d2h_bytes_per_step": int(cells * host.itemsize / shots),
               "shots": shots, "host_buffers": "pinned (page-locked) input and output arrays",
               "calls": reps, "call_ms": pipe_ms,
               "copies": "overlapped: set_psi_async / get_psi_async on copy streams beside the steps",
               "serial": {"value": world * cells * shots * reps / et, "call_ms": call_ms, "call_parts": parts},
               "pipelined_equals_serial": same,
               "note": "per call: H2D of the state + shots RK3 steps + diag + D2H of the state, every copy inside "
                       "the timed region; 'value' overlaps the copies with the steps, 'serial' runs set_psi, "
                       "step_rt, diag, get_psi one after another; one untimed call of each first"}

    # ---- precision: FP32 (three stages and compensated) against FP64 -----------
    # The same start advanced `precision_steps` steps with the same Omega ramp in
    # the plain FP32 form, the compensated FP32 form and FP64; the FP64 run is
    # also the FP64 throughput line.
    fp64 = None
    comp = None
    other_forms = {}
    precision = None
    if not args.no_fp64 and prec == abi.FP32:
        import numpy as np
        start = ground[0] if ground is not None else None
        if start is None:
            s.init_state(init["name"], seed=init["seed"] + rank, amp=init["amp"], r_tf2=init["r_tf2"],
                         noise_amp=init["noise_amp"])
            start = s.get_psi()
        P = args.precision_steps
        runs = {}

        def run_form(sol, form_tag):
            sol.set_psi(start if form_tag != "fp64" else start.astype(np.complex128))
            sol.set_scalar(abi.SCALAR_T, 0.0)
            dstart = sol.diag()
            timed_steps(sol, 2, chunk, omega_of_step, 0)          # warm-up, then the same start again
            sol.set_psi(start if form_tag != "fp64" else start.astype(np.complex128))
            sol.set_scalar(abi.SCALAR_T, 0.0)
            ms_, _ = timed_steps(sol, P, chunk, omega_of_step, 0)
            runs[form_tag] = (dstart, sol.diag(), sol.get_psi().astype(np.complex128), ms_)

        # every FP32 form from the same start, each on its own autotuned tile shape
        form_runs = {}
        for form, tag in ((abi.RK3_THREE_STAGE, "fp32"), (abi.RK3_COMPENSATED, "fp32_compensated"),
                          (abi.RK3_PSI_DIFF, "fp32_psi_diff")):
            s.set_stage_form(form)
            tune_f = None if args.no_autotune or args.kernel else s.autotune(steps=4)
            run_form(s, tag)
            form_runs[form] = {"tag": tag, "autotune": tune_f, "tile": list(s.tile_shape(real_time=True)),
                               "ran": s.stage_form() == form}
        s.close()
        prob64, _ = make_problem(n, abi.FP64)
        s64 = Solver(prob64.to_params())
        if not args.no_autotune:
            s64.autotune(steps=2)
        run_form(s64, "fp64")
        s64.close()
        d64s, d64e, psi64, ms64 = runs["fp64"]

        # States are compared through the raw sums (no cell volume): an FP32
        # context forms h, and so dV, in FP32 as the reference's FP32 build
        # does, which alone puts ~6e-8 between the two precisions' norms.
        def raw_energy(d):
            return -0.5 * d["kinetic"] + 0.5 * d["potential"] + 0.25 * d["interaction"] - 0.5 * d["rotation"]

        def versus(tag):
            ds, de, psi, _ = runs[tag]
            return {"norm_rel": de["intpsi2"] / d64e["intpsi2"] - 1.0,
                    "energy_rel": raw_energy(de) / raw_energy(d64e) - 1.0,
                    "l2_rel_psi": float(np.linalg.norm((psi - psi64).ravel()) / np.linalg.norm(psi64.ravel())),
                    "norm_drift": de["norm"] / ds["norm"] - 1.0, "energy_drift": de["energy"] / ds["energy"] - 1.0}

        precision = {
            "steps": P, "start": ("ground state at Omega = 0 (imaginary time, FP32 state, FP64 renormalisation)"
                                  if ground is not None else "TF cloud + 1e-2 noise"),
            "unit_scale": "Thomas-Fermi mu = 0.4608 (the state's own mu differs by ~0.8%: it turns slowly in phase)",
            "compared": "sum |psi|^2 and the energy's raw sums (no cell volume) after `steps` steps, FP32 / FP64 - 1; "
                        "L2 of psi relative to FP64; drifts relative to each run's own start",
            "fp32": versus("fp32"), "fp32_compensated": versus("fp32_compensated"),
            "fp32_psi_diff": versus("fp32_psi_diff"),
            "headline_form": {abi.RK3_THREE_STAGE: "fp32", abi.RK3_COMPENSATED: "fp32_compensated",
                              abi.RK3_PSI_DIFF: "fp32_psi_diff"}.get(form_run),
            "fp64_drift": {"norm": d64e["norm"] / d64s["norm"] - 1.0, "energy": d64e["energy"] / d64s["energy"] - 1.0},
        }
        def form_line(form):
            fr = form_runs[form]
            msf = runs[fr["tag"]][3]
            ach_f = cells * P * ALG_BYTES[form] / (msf * 1e-3) / 1e9
            ach_m = cells * P * FORM_BYTES[form] / (msf * 1e-3) / 1e9
            return {"value": cells * P / (msf * 1e-3), "unit": UNIT, "ms_per_step": msf / P, "steps": P,
                    "tile": fr["tile"], "autotune": fr["autotune"], "ran": fr["ran"],
                    "roofline": {"bound": "hbm", "achieved": ach_f, "peak": peak, "unit": "GB/s",
                                 "frac": ach_f / peak, "algorithmic_bytes_per_point_step": ALG_BYTES[form],
                                 "form_bytes_per_point_step": FORM_BYTES[form], "frac_of_form_bytes": ach_m / peak,
                                 "traffic": (lambda t: t * cells if t else None)(
                                     profile_traffic("fp32", *fr["tile"], form=FORM_PROFILE.get(form, "")))},
                    "rk3_form": FORM_TEXT[form]}

        comp = form_line(abi.RK3_COMPENSATED)
        # the form of the timed run is the headline; the other plain forms are reported beside it
        other_forms = {f: form_line(f) for f in (abi.RK3_THREE_STAGE, abi.RK3_PSI_DIFF) if f != form_run}
        v64 = cells * P / (ms64 * 1e-3)
        fma = fp64_fma_peak()
        fp64 = {"value": v64, "unit": UNIT, "ms_per_step": ms64 / P,
                "hbm_gbs_alg": cells * P * 160.0 / (ms64 * 1e-3) / 1e9,
                "hbm_frac": cells * P * 160.0 / (ms64 * 1e-3) / 1e9 / peak,
                "compute_roofline": {"bound": "fp64", "ops_per_point_step": FP64_OPS_PER_POINT_STEP,
                                     "achieved": v64 * FP64_OPS_PER_POINT_STEP / 1e12,
                                     "peak": fma / 1e12, "unit": "T FP64 instructions/s",
                                     "frac": v64 * FP64_OPS_PER_POINT_STEP / fma,
                                     "peak_kind": "measured: trapbec_fp64_fma_rate (FMA chains on every SM)"},
                "note": "FP64 stage kernels are bound by GB300's FP64 pipe, not HBM"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        k_cpu = max(1, args.cpu_steps)
        val, cores, dt = cpu_reference(n, k_cpu, None)
        cpu = {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{k_cpu} RK3 steps of the full {n}^3 FP32 grid on the host cores ({dt:.1f} s)"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 (f32)" if prec == abi.FP32 else "c128 (f64)",
        "data": ("synthetic: the seeded TF cloud + 1e-2 noise relaxed to the ground state at Omega = 0 in "
                 "imaginary time on the GPU" if ground is not None else
                 "synthetic (seeded TF cloud + 1e-2 noise standing in for the relaxed ground state)"),
        "config": {"workload": f"rotating-trap RK3 quench {n}^3 complex {'FP32' if prec == abi.FP32 else 'FP64'}",
                   "grid": [n, n, n], "box": [128.0, 128.0, 128.0], "dt_trap_units": 0.004,
                   "omega_ramp": "0 -> 0.8 omega_perp over 5000 steps, updated every chunk",
                   "chunk_steps": chunk, "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2_flush": "inputs larger than L2 (1 GiB per array)",
                   "kernel": kernel_name, "tile": [tz_run, ty_run], "autotune": tune,
                   "rk3_form": FORM_TEXT[form_run]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_point_step": bpc,
                     "form_bytes_per_point_step": fbc, "frac_of_form_bytes": achieved_form / peak,
                     "kernel": "stage_tiled_kernel (3 launches per RK3 step; achieved averaged over them)"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "wall_s_timed": wall,
        "drift": {"norm_rel": d1["norm"] / d0["norm"] - 1.0, "energy_rel": d1["energy"] / d0["energy"] - 1.0,
                  "steps": args.warmup + args.steps, "note": "the FP32 run's own change over its warm-up and timed steps"},
    }
    if ground is not None:
        line["start"] = {"imag_steps": ground[1], "imag_rel_dE": ground[2], "imag_ms_device": ground[3],
                         "dtau_trap_units": ground[4]}
    if precision:
        line["fp32_vs_fp64"] = precision
    if comp:
        line["compensated"] = comp
    for f, v in other_forms.items():
        line[{abi.RK3_THREE_STAGE: "three_stage", abi.RK3_PSI_DIFF: "psi_diff"}[f]] = v
    if fp64:
        line["fp64"] = fp64
    if not args.no_stretch and rank == 0 and world == 1 and n == 512:
        line["stretch_1024"] = stretch_leg(args, peak)
    if not args.no_ring and rank == 0 and world == 1:
        line["ring256"] = ring_leg(args, peak)
    if not args.no_imag and rank == 0 and world == 1:
        line["imag"] = imag_leg(args)
    if rank == 0 and world == 1 and not args.no_warmstart:
        line["warmstart"] = warmstart_leg(args)
        line["warmstart"]["surrogate_kernels"] = surrogate_kernels()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=512, help="grid size per axis (profiling uses smaller cases)")
    ap.add_argument("--chunk", type=int, default=20, help="RK3 steps per C-ABI call (Omega updated per call)")
    ap.add_argument("--shots", type=int, default=100, help="RK3 steps per end-to-end call")
    ap.add_argument("--e2e-reps", type=int, default=10, help="timed end-to-end calls (after one untimed call)")
    ap.add_argument("--precision-steps", type=int, default=500,
                    help="steps of the FP32 / compensated FP32 / FP64 comparison from the same start")
    ap.add_argument("--start", default="ground", choices=["ground", "tf"],
                    help="start of the 512^3 run: the imaginary-time ground state or the TF + noise cloud")
    ap.add_argument("--cpu-steps", type=int, default=12, help="RK3 steps of the CPU baseline sample")
    ap.add_argument("--fp64-only", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--kernel", type=int, nargs=3, default=None, metavar=("KIND", "TZ", "TY"))
    ap.add_argument("--no-autotune", action="store_true", help="keep the default tile shape and work order")
    ap.add_argument("--work-chunk", type=int, default=None,
                    help="work order of the timed run's tiled kernel (trapbec_set_chunk; < 0: strided order)")
    ap.add_argument("--stage-form", type=int, default=3, choices=[0, 1, 2, 3],
                    help="real-time RK3 form of the timed run: 0 three full stages, 1 deferred psi1 "
                         "(stage 1 stores w1 only), 2 compensated state, 3 psi difference (no w array)")
    ap.add_argument("--no-ring", action="store_true", help="skip the 256^3 vortex-ring FP32/FP64 leg")
    ap.add_argument("--no-stretch", action="store_true", help="skip the 1024^3 stretch leg")
    ap.add_argument("--stretch-steps", type=int, default=60)
    ap.add_argument("--ring-steps", type=int, default=2000)
    ap.add_argument("--no-imag", action="store_true", help="skip the batched imaginary-time leg")
    ap.add_argument("--imag-count", type=int, default=64)
    ap.add_argument("--imag-seed", type=int, default=3)
    ap.add_argument("--imag-grids", type=int, nargs="+", default=[64, 96, 128])
    ap.add_argument("--imag-tol", type=float, default=1e-10)
    ap.add_argument("--imag-max-steps", type=int, default=20000)
    ap.add_argument("--no-warmstart", action="store_true", help="skip the NN-vs-TF imaginary-time leg")
    ap.add_argument("--ws-count", type=int, default=16, help="held-out draws of the NN-vs-TF leg")
    ap.add_argument("--ws-max-steps", type=int, default=20000)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    from trapbec_gb300.build import build_library
    build_library()
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
