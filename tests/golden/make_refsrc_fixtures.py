"""Generate tests/golden/refsrc_cases.{json,npz}: golden vectors produced by
the reference's own Fortran source, executed by oracle/fortran_subset.py
(oracle/refsrc.py runs `program run` of src/run.f90 with the modules it uses,
on 1 rank or a 2 x 2 grid of virtual MPI ranks, FP32 as shipped and the FP64
build).

Run in a checkout where the reference's sources are present:
    python tests/golden/make_refsrc_fixtures.py --ref-src /root/reference/src

Each case records the trapbec_params it was run with, the start state (where
it came through the restart files), the state the reference wrote after the
last step (var0001.dat, gathered over ranks), rank 0's standard output and,
where switched on, the vel01.dat / qpress01.dat diagnostics; for a few
single-rank cases the raw bytes of the unformatted files the reference wrote
(tests/golden/refsrc_files.npz).  The fixtures are read by
tests/test_refsrc_golden.py (the oracle, CPU) and tests/test_gpu_refsrc.py
(the CUDA path and this library's writers).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import struct
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refbin_parity as rb  # noqa: E402
from oracle import refsrc  # noqa: E402
from tests.helpers import params, smooth_state  # noqa: E402
from trapbec_gb300 import abi, units  # noqa: E402

PARAM_FIELDS = ("nx", "ny", "nz", "lx", "ly", "lz", "precision", "boundaries", "periodicz", "two_dim", "potential",
                "lbeam", "winding_number", "vor_ring_count", "dt_re", "dt_im", "gamma", "harm_wx", "harm_wy",
                "harm_wz", "potential_off", "wbeam", "advective_vx", "omega_z", "t_spindown", "ring_rad",
                "nprocx", "nprocy")


def _pdict(p):
    return {f: getattr(p, f) for f in PARAM_FIELDS}


def _line16(prec, nproc):
    """The 64^3 vortex-line workload (TF x Pade line, isotropic trap) on a
    16^3 grid of the same spacing (dx = 0.5)."""
    prob, init = units.vortex_line_64(prec, nproc=nproc)
    p = prob.to_params()
    p.nx = p.ny = p.nz = 16
    p.lx = p.ly = p.lz = p.lx / 4
    p64 = prob.to_params()
    p64.nx = p64.ny = p64.nz = 16
    p64.lx = p64.ly = p64.lz = p64.lx / 4
    p64.precision = abi.FP64
    psi0 = rb.start_state(p64, init)
    return p, psi0


def _read_field(datadir, name, n, nprocs, fp64):
    """vel01.dat / qpress01.dat of every rank: coords(2) int32 then the
    (nz, ny, nx, 3) real array (src/output.f90:77-91), as (3, Nx, Ny, Nz)."""
    dims = rb.mpi_dims_create(nprocs)
    nx, ny, nz = n
    mx, my = nx // dims[0], ny // dims[1]
    dt = np.float64 if fp64 else np.float32
    out = np.zeros((3, nx, ny, nz), dtype=dt)
    for r in range(nprocs):
        rec = rb._read_records(os.path.join(datadir, "proc%03d" % r, name))[0]
        cx, cy = struct.unpack("<2i", rec[:8])
        blk = np.frombuffer(rec[8:], dtype=dt).reshape((3, mx, my, nz))
        out[:, cx * mx:(cx + 1) * mx, cy * my:(cy + 1) * my, :] = blk
    return out


def cases():
    """(name, params, start state or None, steps, nprocs, cparam overrides, extra)."""
    out = []
    for prec in (abi.FP64, abi.FP32):
        tag = "fp64" if prec == abi.FP64 else "fp32"
        # the vortex-line workload, 1 rank and 2 x 2 ranks
        for nproc in ((1, 1), (2, 2)):
            p, psi0 = _line16(prec, nproc)
            out.append((f"line16_np{nproc[0] * nproc[1]}_{tag}", p, psi0, 12, nproc[0] * nproc[1], {}, {}))
        # rotating anisotropic trap, 2 x 2 ranks
        p = params(n=(12, 16, 8), L=(6.0, 8.0, 4.0), prec=prec, pot="harmonic", harm=(3.0, 4.0, 5.0), omega=0.3,
                   dt=0.01, nproc=(2, 2))
        out.append((f"rot_np4_{tag}", p, smooth_state(p, seed=41), 6, 4, {}, {}))
        # boundary types on 2 x 2 ranks
        p = params(n=(12, 12, 8), L=(6.0, 6.0, 4.0), prec=prec, bc=abi.BC_SOLID, pot="harmonic",
                   harm=(2.0, 3.0, 4.0), periodicz=1, dt=0.01, nproc=(2, 2))
        out.append((f"solid_pz_np4_{tag}", p, smooth_state(p, seed=42), 5, 4, {}, {}))
        p = params(n=(12, 12, 8), L=(6.0, 6.0, 4.0), prec=prec, bc=abi.BC_PERIODIC, pot="zero", dt=0.01,
                   nproc=(2, 2))
        out.append((f"periodic_np4_{tag}", p, smooth_state(p, seed=43), 5, 4, {}, {}))
        # advective frame
        p = params(n=(12, 12, 8), L=(6.0, 6.0, 4.0), prec=prec, pot="zero", periodicz=1, vx=0.25, dt=0.01)
        out.append((f"advective_{tag}", p, smooth_state(p, seed=44), 5, 1, {}, {}))
    # the vortex-line workload at its own size (64^3 on [-16, 16]^3), 3 steps, 1 rank; only a
    # seeded sample of 4096 cells of the final state is kept (with the printed diagnostics line)
    prob, init = units.vortex_line_64(abi.FP64)
    p = prob.to_params()
    psi0 = rb.start_state(p, init)
    out.append(("line64_np1_fp64", p, psi0, 3, 1, {}, {"sample": 4096, "start": "tf_vortex_line"}))
    # other process grids: 2 ranks (MPI_DIMS_CREATE gives 2 x 1) and 8 ranks (4 x 2)
    for nprocs in (2, 8):
        dims = rb.mpi_dims_create(nprocs)
        p, psi0 = _line16(abi.FP64, dims)
        out.append((f"line16_np{nprocs}_fp64", p, psi0, 6, nprocs, {}, {}))
    # the time switches of get_rhs: the potential off after potential_off (finite_diff.f90:124) and
    # the rotating frame off after t_spindown (finite_diff.f90:128), both inside the run
    p = params(n=(12, 12, 8), L=(6.0, 6.0, 4.0), prec=abi.FP64, pot="harmonic", harm=(3.0, 4.0, 5.0), omega=0.3,
               dt=0.01)
    p.potential_off = 0.015
    p.t_spindown = 0.025
    out.append(("switches_fp64", p, smooth_state(p, seed=50), 4, 1, {}, {}))
    # the potential library and the laser, FP64, 1 rank
    pots = [("barrier", dict(gamma=0.01, dt=0.02, bc=abi.BC_SOLID)), ("box_trap", {}), ("channel", {}),
            ("quartic", dict(harm=(900.0, 8.0, 6.0))), ("sphere", {}), ("harmonic_ring", dict(harm=(50.0, 0, 0))),
            ("harmonic", dict(lbeam=1, harm=(3.0, 4.0, 5.0)))]
    for pot, kw in pots:
        kw = dict(kw)
        dt = kw.pop("dt", 0.01)
        p = params(n=(12, 12, 8), L=(24.0, 24.0, 16.0), prec=abi.FP64, pot=pot, dt=dt, **kw)
        nm = f"pot_{pot}{'_lbeam' if kw.get('lbeam') else ''}_fp64"
        out.append((nm, p, smooth_state(p, seed=45), 3, 1, {}, {}))
    # the set-up of the reference's own cparam.local (src/cparam.local:1-44): a 2D run (Nz = 1,
    # two_dim, periodic z) in a quartic trap with the laser, FP32 as shipped and FP64; and the
    # second ring potential
    for prec in (abi.FP32, abi.FP64):
        p = params(n=(16, 16, 1), L=(32.0, 32.0, 1.0), prec=prec, pot="quartic", harm=(900.0, 8.0, 6.0),
                   periodicz=1, two_dim=1, lbeam=1, gamma=0.003, dt=0.01, nproc=(2, 2))
        tag = "fp64" if prec == abi.FP64 else "fp32"
        out.append((f"sample2d_np4_{tag}", p, smooth_state(p, seed=48), 4, 4, {}, {}))
    p = params(n=(12, 12, 8), L=(24.0, 24.0, 16.0), prec=abi.FP64, pot="harmonic_ring2", dt=0.01)
    out.append(("pot_harmonic_ring2_fp64", p, smooth_state(p, seed=49), 3, 1, {}, {}))
    # the 'mobius' potential, whose Trap array mesh_init builds (initial.f90:159-198) -- only when the
    # run does not restart, so these start from init_cond 'constant' -- a 200 x 200 sum per cell, so a
    # small grid; 1 rank and 2 x 2 ranks (the Trap's maximum over the ranks)
    for nproc, prec in (((1, 1), abi.FP64), ((2, 2), abi.FP64), ((1, 1), abi.FP32)):
        p = params(n=(8, 8, 6), L=(64.0, 64.0, 16.0), prec=prec, pot="mobius", dt=0.01, nproc=nproc)
        tag = "fp64" if prec == abi.FP64 else "fp32"
        out.append((f"pot_mobius_np{nproc[0] * nproc[1]}_{tag}", p, None, 2, nproc[0] * nproc[1],
                    {"init_cond": "'constant'"}, {"init": "constant"}))
    # imaginary-time Euler (run.f90:19-35) from a reference init_cond, then one RK3 step
    p = params(n=(12, 12, 8), L=(12.0, 12.0, 8.0), prec=abi.FP64, pot="harmonic", harm=(4.0, 4.0, 4.0), dt=0.01)
    p.winding_number = 1
    out.append(("imag_euler_fp64", p, None, 1, 1,
                {"init_cond": "'single_vortex'", "imaginary_time": ".true.", "imag_nsteps": "6"},
                {"imag_steps": 6}))
    # imaginary time with the phase imprint after every step (run.f90:26) and the imag_var files
    # (output.f90:55-62), from single_vortex; checked through the program-run driver
    p = params(n=(12, 12, 8), L=(12.0, 12.0, 8.0), prec=abi.FP64, pot="harmonic", harm=(4.0, 4.0, 4.0), dt=0.01)
    p.winding_number = 2
    out.append(("imag_imprint_fp64", p, None, 1, 1,
                {"init_cond": "'single_vortex'", "imaginary_time": ".true.", "imag_nsteps": "4",
                 "phase_imprint_on": ".true.", "imaginary_output": ".true."},
                {"imag_steps": 4, "imag_file": True}))
    # the init_cond library: dt = 0, one step, so var0001.dat holds the initial state
    for ic, extra_p in (("constant", {}), ("soliton", {}), ("single_vortex", {"winding_number": 2}),
                        ("sausage", {}), ("crow", {}), ("leap_frog", {}), ("line_of_lines", {"ring_rad": 4.0}),
                        ("linked_rings", {"ring_rad": 4.0}), ("lattice2", {}), ("bundle", {})):
        p = params(n=(12, 12, 8), L=(40.0, 40.0, 24.0), prec=abi.FP64, pot="harmonic", harm=(3.0, 4.0, 5.0),
                   dt=0.0)
        for k, v in extra_p.items():
            setattr(p, k, v)
        out.append((f"init_{ic}_fp64", p, None, 1, 1, {"init_cond": f"'{ic}'"}, {"init": ic}))
    # helpers applied by program run after the initial state (run.f90:37-40)
    for helper, flag in (("add_ring", "add_ring"), ("add_dipole", "add_dipole"), ("add_pcurrent", "add_pcurrent")):
        pot = "barrier" if helper == "add_pcurrent" else "harmonic"
        p = params(n=(12, 12, 8), L=(48.0, 48.0, 24.0), prec=abi.FP64, pot=pot, harm=(3.0, 4.0, 5.0), dt=0.0)
        p.ring_rad = 5.0
        out.append((f"helper_{helper}_fp64", p, None, 1, 1, {"init_cond": "'constant'", flag: ".true."},
                    {"init": "constant", "helper": helper}))
    # output-time diagnostics: get_phase velocity and quantum pressure (vel01.dat, qpress01.dat)
    for nproc in ((1, 1), (2, 2)):
        p = params(n=(12, 12, 8), L=(6.0, 6.0, 4.0), prec=abi.FP64, pot="harmonic", harm=(2.0, 3.0, 4.0),
                   omega=0.2, dt=0.01, nproc=nproc)
        out.append((f"diag_np{nproc[0] * nproc[1]}_fp64", p, smooth_state(p, seed=46), 2, nproc[0] * nproc[1],
                    {"vel_print": ".true.", "qpress_print": ".true."}, {"diag": True}))
    return out


# Cases whose output files are also kept byte for byte (tests/golden/refsrc_files.npz):
# the unformatted records var_print writes (src/output.f90:64-75,80-91,102-108) on 1 rank.
FILE_CASES = {"line16_np1_fp64": ("var0001.dat", "var.dat"), "line16_np1_fp32": ("var0001.dat", "var.dat"),
              "diag_np1_fp64": ("var0001.dat", "var.dat", "vel01.dat", "qpress01.dat")}


def write_file_fixtures(ref_src) -> None:
    """Run the FILE_CASES again and keep the raw bytes of the files the
    reference wrote into data/proc000 (tests/golden/refsrc_files.npz)."""
    import shutil
    out = {}
    for name, p, psi0, steps, nprocs, over, extra in cases():
        if name not in FILE_CASES:
            continue
        keep = os.path.join("/tmp", f"refsrc_files_{name}")
        shutil.rmtree(keep, ignore_errors=True)
        os.makedirs(keep)
        refsrc.run_reference(ref_src, p, psi0, steps, nprocs, p.precision == abi.FP64, cparam_overrides=over,
                             keep=keep)
        for f in FILE_CASES[name]:
            data = open(os.path.join(keep, "data", "proc000", f), "rb").read()
            out[f"{name}__{f}"] = np.frombuffer(data, dtype=np.uint8)
        shutil.rmtree(keep, ignore_errors=True)
        print(f"{name}: files kept", flush=True)
    np.savez_compressed(os.path.join(HERE, "refsrc_files.npz"), **out)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--ref-src", default="/root/reference/src")
    ap.add_argument("--only", default=None, help="substring of the case names to run")
    ap.add_argument("--files-only", action="store_true", help="only refsrc_files.npz")
    ap.add_argument("--merge", action="store_true",
                    help="with --only: add the selected cases to the existing fixtures instead of discarding them")
    args = ap.parse_args(argv)
    if args.files_only:
        write_file_fixtures(args.ref_src)
        return 0
    meta = {"generator": "tests/golden/make_refsrc_fixtures.py",
            "interpreter": "oracle/fortran_subset.py (gfortran -O3 x86-64 semantics, no FP contraction)",
            # the intrinsic functions come from this machine's libm (hypot, expf, ...)
            "platform": {"machine": platform.machine(), "libc": " ".join(platform.libc_ver())},
            "cases": {}}
    arrays = {}
    for name, p, psi0, steps, nprocs, over, extra in cases():
        if args.only and args.only not in name:
            continue
        fp64 = p.precision == abi.FP64
        t0 = time.time()
        keep = os.path.join("/tmp", f"refsrc_{name}")
        import shutil
        shutil.rmtree(keep, ignore_errors=True)
        os.makedirs(keep)
        r = refsrc.run_reference(args.ref_src, p, psi0, steps, nprocs, fp64, cparam_overrides=over, keep=keep)
        rec = {"params": _pdict(p), "steps": steps, "nprocs": nprocs, "dims": list(r["dims"]), "t": r["t"],
               "cparam_overrides": over, "stdout": r["stdout"], "seconds": round(time.time() - t0, 1)}
        rec.update(extra)
        if extra.get("sample"):
            # large grid: the start state is the workload's own (rebuilt by the tests), and the
            # final state is kept at a seeded sample of cells
            idx = np.sort(np.random.default_rng(7).choice(r["psi"].size, extra["sample"], replace=False))
            arrays[f"{name}__idx"] = idx
            arrays[f"{name}__psi_sample"] = r["psi"].ravel()[idx]
        else:
            if psi0 is not None:
                arrays[f"{name}__psi0"] = psi0.astype(np.complex128 if fp64 else np.complex64)
            arrays[f"{name}__psi"] = r["psi"]
        if extra.get("imag_file"):
            # the last imag_var####.dat (itime/shots = imag_steps with shots = 1), rank 0's record
            _, _, blk = rb.read_var(os.path.join(keep, "data", "proc000", "imag_var%04d.dat" % extra["imag_steps"]),
                                    (p.nx, p.ny, p.nz), fp64)
            arrays[f"{name}__psi_imag"] = np.array(blk)
        if extra.get("diag"):
            n = (p.nx, p.ny, p.nz)
            arrays[f"{name}__vel"] = _read_field(os.path.join(keep, "data"), "vel01.dat", n, nprocs, fp64)
            arrays[f"{name}__qpress"] = _read_field(os.path.join(keep, "data"), "qpress01.dat", n, nprocs, fp64)
        shutil.rmtree(keep, ignore_errors=True)
        meta["cases"][name] = rec
        print(f"{name}: {rec['seconds']} s", flush=True)
    if args.only and args.merge:
        old_meta = json.load(open(os.path.join(HERE, "refsrc_cases.json")))
        old_arrays = dict(np.load(os.path.join(HERE, "refsrc_cases.npz")))
        old_meta["cases"].update(meta["cases"])
        old_arrays.update(arrays)
        np.savez_compressed(os.path.join(HERE, "refsrc_cases.npz"), **old_arrays)
        with open(os.path.join(HERE, "refsrc_cases.json"), "w") as f:
            json.dump(old_meta, f, indent=1, default=float)
    if not args.only:
        np.savez_compressed(os.path.join(HERE, "refsrc_cases.npz"), **arrays)
        with open(os.path.join(HERE, "refsrc_cases.json"), "w") as f:
            json.dump(meta, f, indent=1, default=float)
        write_file_fixtures(args.ref_src)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
