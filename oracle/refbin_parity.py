"""Reference-binary parity harness (test infrastructure, not product code).

Builds the reference program (Fortran 90 + MPI) from its own source files,
runs a workload through the reference's restart path, gathers the var####.dat
files it writes and compares them with the oracle (the CPU restatement of the
reference in oracle/trapbec_oracle.cpp) after the same number of steps.  This
is the only way to tie the oracle, and through it the GPU path, to the
reference itself.

It needs a Fortran compiler with MPI: `mpif90` and `mpiexec` on PATH.
Neither this project's build image nor its GPU hosts have them, so there
`available()` returns False with the reason and the tests that would run the
binary skip; every step up to the compiler call (parameter file, per-rank
restart files, the FP64 source patch, the gather of the output) is covered by
tests/test_refbin_harness.py without it.

Steps, with the reference lines each one follows:
 1. cparam.local of the workload (the full set of names run.f90 needs, in the
    syntax of src/cparam.local:1-44): the trap-units workload mapped onto
    the reference's units by trapbec_gb300/units.py, `imaginary_time` off,
    `full_binary_output` on, `shots`/`nsteps` so that output lands at the
    steps compared.
 2. The start state as restart files: data/proc%02d/var.dat per rank (the
    reader's i2.2 directory, src/initial.f90:44,800) with the three records
    itime, t, Psi(1:nmeshz,1:nmeshy,1:nmeshx) of src/initial.f90:796-818 and
    src/output.f90:103-108; itime = 1 so that the time loop
    `do itime=nstart,nsteps` (src/run.f90:43) runs `nsteps` steps.  The
    writer's i3.3 directories data/proc%03d (src/output.f90:73,103) are
    created for the output.  Rank r of the MPI_CART_CREATE grid has coords
    (r / dims(2), r mod dims(2)) and owns x block coords(1), y block coords(2)
    (src/mpi_var.f90:27-37).
 3. Build: `mpif90 -O3` on each source in dependency order (the flags of
    src/Makefile:1-2) for the shipped single precision; for the FP64 run the
    same with `-fdefault-real-8 -fdefault-double-8` after replacing the
    hard-coded MPI_COMPLEX and MPI_REAL of src/ghost.f90,
    src/diagnostic.f90, src/initial.f90 and src/force.f90 with
    MPI_DOUBLE_COMPLEX and MPI_DOUBLE_PRECISION (without the patch a
    multi-rank FP64 run exchanges half of each halo plane).  The sources are
    copied into a scratch directory; the reference tree is only read.
 4. Run: `mpiexec -n P ./run.x` (run.sh:37).
 5. Gather: data/proc%03d/var%04d.dat, one record coords(2) int32, Lx, Ly,
    Lz, t (reals of the build's kind), Psi (bin/gather.m:6-28).
 6. Compare with the oracle on the same process grid after the same steps:
    FP64 to 1e-12 relative in psi, norm and energy; FP32 at FP32 rounding.

Usage (on a host with mpif90 and mpiexec):
    python -m oracle.refbin_parity --ref-src /root/reference/src [--work DIR]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import shutil
import struct
import subprocess
import sys
import tempfile

import numpy as np

# dependency order of the reference's modules (src/Makefile:33-56), run.f90 last
SOURCES = ["cdata.f90", "mpi_var.f90", "statistics.f90", "initial.f90", "ghost.f90", "deriv.f90",
           "finite_diff.f90", "output.f90", "diagnostic.f90", "force.f90"]
MAIN = "run.f90"
FFLAGS = ["-O3"]
FFLAGS_FP64 = ["-O3", "-fdefault-real-8", "-fdefault-double-8"]


def toolchain() -> dict:
    return {"mpif90": shutil.which("mpif90"), "mpiexec": shutil.which("mpiexec")}


def available() -> tuple[bool, str]:
    t = toolchain()
    missing = [k for k, v in t.items() if not v]
    if missing:
        return False, "no " + " / ".join(missing) + " on this machine: the reference (Fortran 90 + MPI) cannot be built"
    return True, ""


def mpi_dims_create(nprocs: int) -> tuple[int, int]:
    """The balanced 2-D factorisation MPI_DIMS_CREATE returns for an empty
    dims array (src/mpi_var.f90:24): factors as close as possible, in
    non-increasing order."""
    best = (nprocs, 1)
    for a in range(1, int(math.isqrt(nprocs)) + 1):
        if nprocs % a == 0:
            b = nprocs // a
            best = (max(a, b), min(a, b))
    return best


def rank_coords(rank: int, dims: tuple[int, int]) -> tuple[int, int]:
    """MPI_CART_COORDS of a row-major Cartesian communicator."""
    return rank // dims[1], rank % dims[1]


# ---- 1. cparam.local --------------------------------------------------------
def _real(v: float) -> str:
    if v >= 3.0e38:
        return "huge(1.)"
    s = repr(float(v))
    return s if ("." in s or "e" in s or "inf" in s) else s + "."


def _logical(b) -> str:
    return ".true." if b else ".false."


def cparam_text(p, nsteps: int, shots: int) -> str:
    """A complete cparam.local for trapbec_params `p` (the names and types of
    src/cparam.local:1-44)."""
    pots = ["zero", "harmonic", "harmonic_ring", "harmonic_ring2", "barrier", "box_trap", "channel", "quartic",
            "sphere", "mobius", "array"]
    bcs = ["zero", "solid", "periodic"]
    lines = [
        "!/* generated by oracle/refbin_parity.py */",
        f"real  :: Lx={_real(p.lx)}, Ly={_real(p.ly)}, Lz={_real(p.lz)}",
        f"integer, parameter :: Nx={p.nx}, Ny={p.ny}, Nz={p.nz}",
        f"complex :: dt=({_real(p.dt_re)},{_real(p.dt_im)})",
        f"integer, parameter :: shots={shots}",
        f"integer, parameter :: nsteps={nsteps}",
        f"character(len=*), parameter :: boundaries='{bcs[p.boundaries]}'",
        f"logical, parameter :: periodicz={_logical(p.periodicz)}",
        "character(len=*), parameter :: init_cond='constant'",
        f"character(len=*), parameter :: potential='{pots[p.potential]}'",
        f"real, parameter :: harm_wx={_real(p.harm_wx)}, harm_wy={_real(p.harm_wy)}, harm_wz={_real(p.harm_wz)}",
        f"real, parameter :: potential_off={_real(p.potential_off)}",
        f"real, parameter :: gamma={_real(p.gamma)}",
        f"logical, parameter :: two_dim={_logical(p.two_dim)}",
        "logical, parameter :: phase_imprint_on=.false.",
        f"logical, parameter :: lbeam={_logical(p.lbeam)}",
        "logical, parameter :: add_pcurrent=.false.",
        f"real, parameter :: wbeam={_real(p.wbeam)}",
        f"real, parameter :: advective_vx={_real(p.advective_vx)}",
        f"real, parameter :: omega_z={_real(p.omega_z)}",
        f"real, parameter :: t_spindown={_real(p.t_spindown)}",
        f"integer, parameter :: winding_number={p.winding_number}",
        f"integer, parameter :: vor_ring_count={p.vor_ring_count}",
        f"real,parameter :: ring_rad={_real(p.ring_rad)}",
        "logical, parameter :: add_ring=.false.",
        "logical, parameter :: add_dipole=.false.",
        "integer, parameter :: vor_line_count=1",
        "logical, parameter :: imaginary_time=.false.",
        "integer, parameter :: imag_nsteps=0",
        "logical, parameter :: forcing=.false.",
        "integer, parameter :: force_freq=10",
        "logical, parameter :: full_binary_output=.true.",
        "logical, parameter :: imaginary_output=.false.",
        "logical, parameter :: gnuplot_2d_print=.false.",
        "logical, parameter :: qpress_print=.false.",
        "logical, parameter :: vel_print=.false.",
    ]
    return "\n".join(lines) + "\n"


# ---- 2. restart files -------------------------------------------------------
def _record(payload: bytes) -> bytes:
    n = struct.pack("<i", len(payload))
    return n + payload + n


def _read_records(path: str) -> list[bytes]:
    data = open(path, "rb").read()
    out, off = [], 0
    while off < len(data):
        n = struct.unpack("<i", data[off:off + 4])[0]
        out.append(data[off + 4:off + 4 + n])
        off += 8 + n
    return out


def split_ranks(psi: np.ndarray, dims: tuple[int, int]) -> list[np.ndarray]:
    """Per-rank blocks of a global psi[x, y, z] (z fastest, the reference's
    Psi(k,j,i) order) in rank order."""
    nx, ny, _ = psi.shape
    mx, my = nx // dims[0], ny // dims[1]
    blocks = []
    for r in range(dims[0] * dims[1]):
        cx, cy = rank_coords(r, dims)
        blocks.append(np.ascontiguousarray(psi[cx * mx:(cx + 1) * mx, cy * my:(cy + 1) * my, :]))
    return blocks


def write_restart(datadir: str, psi: np.ndarray, nprocs: int, fp64: bool, itime: int = 1, t: float = 0.0) -> None:
    """data/proc%02d/var.dat for every rank (src/initial.f90:796-818) and the
    empty output directories data/proc%03d (src/output.f90:73)."""
    dims = mpi_dims_create(nprocs)
    cdt = np.complex128 if fp64 else np.complex64
    for r, blk in enumerate(split_ranks(psi.astype(cdt), dims)):
        d = os.path.join(datadir, "proc%02d" % r)
        os.makedirs(d, exist_ok=True)
        os.makedirs(os.path.join(datadir, "proc%03d" % r), exist_ok=True)
        with open(os.path.join(d, "var.dat"), "wb") as f:
            f.write(_record(struct.pack("<i", itime)))
            f.write(_record(struct.pack("<d" if fp64 else "<f", t)))
            f.write(_record(blk.tobytes()))


def read_restart(path: str, local_shape: tuple[int, int, int], fp64: bool) -> tuple[int, float, np.ndarray]:
    recs = _read_records(path)
    itime = struct.unpack("<i", recs[0])[0]
    t = struct.unpack("<d" if fp64 else "<f", recs[1])[0]
    psi = np.frombuffer(recs[2], dtype=np.complex128 if fp64 else np.complex64).reshape(local_shape)
    return itime, t, psi


# ---- 5. gather ----------------------------------------------------------------
def read_var(path: str, local_shape: tuple[int, int, int], fp64: bool) -> tuple[tuple[int, int], tuple, np.ndarray]:
    """One var####.dat record: coords(2) int32, Lx, Ly, Lz, t, Psi (bin/gather.m:6-28)."""
    rec = _read_records(path)[0]
    rs = 8 if fp64 else 4
    coords = struct.unpack("<2i", rec[:8])
    hdr = struct.unpack("<4d" if fp64 else "<4f", rec[8:8 + 4 * rs])
    psi = np.frombuffer(rec[8 + 4 * rs:], dtype=np.complex128 if fp64 else np.complex64).reshape(local_shape)
    return coords, hdr, psi


def gather(datadir: str, index: int, n: tuple[int, int, int], nprocs: int, fp64: bool) -> tuple[np.ndarray, float]:
    """The global psi of output number `index` from every rank's file, placed
    by the coords each file records; returns (psi, t)."""
    dims = mpi_dims_create(nprocs)
    nx, ny, nz = n
    mx, my = nx // dims[0], ny // dims[1]
    out = np.zeros((nx, ny, nz), dtype=np.complex128 if fp64 else np.complex64)
    t = None
    for r in range(nprocs):
        coords, hdr, blk = read_var(os.path.join(datadir, "proc%03d" % r, "var%04d.dat" % index), (mx, my, nz), fp64)
        out[coords[0] * mx:(coords[0] + 1) * mx, coords[1] * my:(coords[1] + 1) * my, :] = blk
        t = hdr[3]
    return out, t


# ---- 3./4. build and run ------------------------------------------------------
def fp64_patch(src: str) -> str:
    """The hard-coded MPI datatypes of a single-precision build, made double."""
    src = re.sub(r"\bMPI_COMPLEX\b", "MPI_DOUBLE_COMPLEX", src)
    return re.sub(r"\bMPI_REAL\b", "MPI_DOUBLE_PRECISION", src)


def build(ref_src: str, work: str, cparam: str, fp64: bool) -> str:
    tc = toolchain()
    os.makedirs(work, exist_ok=True)
    for name in SOURCES + [MAIN]:
        text = open(os.path.join(ref_src, name)).read()
        if fp64:
            text = fp64_patch(text)
        open(os.path.join(work, name), "w").write(text)
    open(os.path.join(work, "cparam.local"), "w").write(cparam)
    flags = FFLAGS_FP64 if fp64 else FFLAGS
    for name in SOURCES:
        subprocess.run([tc["mpif90"], *flags, "-c", name, "-o", name[:-4] + ".o"], cwd=work, check=True)
    objs = [s[:-4] + ".o" for s in SOURCES]
    subprocess.run([tc["mpif90"], *flags, "-o", "run.x", MAIN, *objs], cwd=work, check=True)
    return os.path.join(work, "run.x")


def run(work: str, nprocs: int, timeout: float = 3600.0) -> subprocess.CompletedProcess:
    tc = toolchain()
    return subprocess.run([tc["mpiexec"], "-n", str(nprocs), "./run.x"], cwd=work, capture_output=True, text=True,
                          timeout=timeout, check=True)


# ---- 6. a workload end to end ----------------------------------------------------
def workloads():
    """(name, trap-units problem, initial state, steps, nprocs) of the two
    workloads the reference can run on CPU: the 64^3 vortex line (1 rank and a
    2x2 process grid) and the 256^3 vortex ring."""
    from trapbec_gb300 import abi, units
    out = []
    for nprocs in (1, 4):
        prob, init = units.vortex_line_64(abi.FP64, nproc=mpi_dims_create(nprocs))
        out.append((f"vortex_line_64_np{nprocs}", prob, init, init["steps"], nprocs))
    prob, init = units.vortex_ring_256(abi.FP64)
    prob.nproc = mpi_dims_create(4)
    out.append(("vortex_ring_256_np4", prob, init, 100, 4))
    return out


def start_state(p, init) -> np.ndarray:
    """The workload's initial state from the oracle (FP64)."""
    from oracle.pyoracle import Oracle
    from trapbec_gb300.abi import InitArgs
    a = InitArgs()
    a.seed = int(init.get("seed", 0))
    a.amp = float(init.get("amp", 1.0))
    for i, v in enumerate(init.get("r_tf2", (0, 0, 0))):
        a.r_tf2[i] = v
    a.ring_radius = float(init.get("ring_radius", 0.0))
    a.core2 = float(init.get("core2", 0.0))
    a.noise_amp = float(init.get("noise_amp", 0.0))
    o = Oracle(p)
    o.init_state(init["name"], a)
    return o.get_psi()


def compare(ref_psi: np.ndarray, p, psi0: np.ndarray, steps: int) -> dict:
    from oracle.pyoracle import Oracle
    o = Oracle(p)
    o.set_psi(psi0)
    o.step_rt(steps)
    b = o.get_psi()
    a = ref_psi.astype(b.dtype)
    na, nb = float(np.sum(np.abs(a) ** 2)), float(np.sum(np.abs(b) ** 2))
    return {"max_rel": float(np.max(np.abs(a - b)) / np.max(np.abs(b))),
            "l2_rel": float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel())),
            "norm_rel": na / nb - 1.0}


def run_workload(ref_src: str, work_root: str, name, prob, init, steps, nprocs, fp64: bool) -> dict:
    from trapbec_gb300 import abi
    prob.precision = abi.FP64 if fp64 else abi.FP32
    p = prob.to_params()
    work = os.path.join(work_root, f"{name}_{'fp64' if fp64 else 'fp32'}")
    build(ref_src, work, cparam_text(p, nsteps=steps, shots=steps), fp64)
    p64 = prob.to_params()
    p64.precision = abi.FP64
    psi0 = start_state(p64, init)
    if not fp64:
        psi0 = psi0.astype(np.complex64)
    write_restart(os.path.join(work, "data"), psi0, nprocs, fp64)
    r = run(work, nprocs)
    ref_psi, t = gather(os.path.join(work, "data"), 1, (p.nx, p.ny, p.nz), nprocs, fp64)
    res = compare(ref_psi, p, psi0, steps)
    res.update({"workload": name, "precision": "fp64" if fp64 else "fp32", "steps": steps, "nprocs": nprocs,
                "t": t, "stdout_tail": r.stdout[-300:]})
    return res


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="parity of the oracle against the reference binary")
    ap.add_argument("--ref-src", default="/root/reference/src")
    ap.add_argument("--work", default=None)
    ap.add_argument("--only", default=None, help="run only the workload of this name")
    a = ap.parse_args(argv)
    ok, why = available()
    if not ok:
        print(json.dumps({"skipped": why}))
        return 0
    work_root = a.work or tempfile.mkdtemp(prefix="refbin_")
    results = []
    for name, prob, init, steps, nprocs in workloads():
        if a.only and name != a.only:
            continue
        for fp64 in (False, True):
            results.append(run_workload(a.ref_src, work_root, name, prob, init, steps, nprocs, fp64))
            print(json.dumps(results[-1]), flush=True)
    bad = [r for r in results if r["max_rel"] > (1e-12 if r["precision"] == "fp64" else 1e-4)]
    return 1 if bad else 0


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.exit(main())
