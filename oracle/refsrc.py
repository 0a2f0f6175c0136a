"""Runs of the reference's own Fortran source through oracle/fortran_subset.py.

Test infrastructure only.  Where no Fortran compiler exists, this takes the
place of the reference binary in the steps of oracle/refbin_parity.py: the
same generated cparam.local (src/cparam.local:1-44), the same per-rank restart
files data/proc%02d/var.dat (src/initial.f90:796-818), the same gather of the
data/proc%03d/var%04d.dat files the reference writes (src/output.f90:64-75,
bin/gather.m:6-28), with `program run` (src/run.f90:1-81) and every module it
uses executed statement by statement by the interpreter, on 1 rank or on a
process grid of virtual MPI ranks.

Only the fixture generator (tests/golden/make_refsrc_fixtures.py) calls
this, where the reference's sources are present; the tests read the
fixtures it writes.
"""
from __future__ import annotations

import os
import shutil
import tempfile

from oracle import fortran_subset as fs
from oracle import refbin_parity as rb


def cparam_for(p, steps: int, shots: int, overrides: dict | None = None) -> str:
    """The cparam.local of oracle/refbin_parity.py for trapbec_params `p`
    with some of its values replaced (name -> Fortran literal)."""
    text = rb.cparam_text(p, nsteps=steps, shots=shots)
    for name, value in (overrides or {}).items():
        lines = text.splitlines()
        for i, ln in enumerate(lines):
            if f":: {name}=" in ln:
                head = ln.split("::")[0]
                lines[i] = f"{head}:: {name}={value}"
                break
        else:
            raise ValueError(f"cparam.local has no {name}")
        text = "\n".join(lines) + "\n"
    return text


def run_reference(ref_src: str, p, psi0, steps: int, nprocs: int, fp64: bool, shots: int | None = None,
                  cparam_overrides: dict | None = None, keep: str | None = None) -> dict:
    """Run the reference's `program run` for `steps` real-time RK3 steps of
    trapbec_params `p` from the global start state `psi0[x, y, z]` (through
    the restart files; None: the cparam's init_cond), on `nprocs` virtual
    ranks, in the FP64 build (`-fdefault-real-8 -fdefault-double-8`) or the
    shipped FP32 one.  Returns the gathered psi of the last output, its t,
    and rank 0's standard output lines."""
    shots = shots or steps
    text = cparam_for(p, steps, shots, cparam_overrides)
    work = keep or tempfile.mkdtemp(prefix="refsrc_")
    try:
        datadir = os.path.join(work, "data")
        os.makedirs(datadir, exist_ok=True)
        dims = rb.mpi_dims_create(nprocs)
        for r in range(nprocs):
            os.makedirs(os.path.join(datadir, "proc%03d" % r), exist_ok=True)
        if psi0 is not None:
            rb.write_restart(datadir, psi0, nprocs, fp64)
        includes = {"cparam.local": text, "mpif.h": fs.MPIF_H}
        ranks = fs.run(ref_src, rb.SOURCES + [rb.MAIN], includes, nprocs, 8 if fp64 else 4, work)
        n = (p.nx, p.ny, p.nz)
        psi, t = rb.gather(datadir, steps // shots, n, nprocs, fp64)
        return {"psi": psi, "t": t, "stdout": list(ranks[0].stdout), "dims": dims, "cparam": text}
    finally:
        if keep is None:
            shutil.rmtree(work, ignore_errors=True)
