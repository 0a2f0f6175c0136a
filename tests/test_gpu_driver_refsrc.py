"""The C++ `program run` equivalent (trapbec_gb300/lib/trapbec_run) against
the reference's own `program run`, end to end.

For every single-rank case of tests/golden/refsrc_cases.* the driver gets
the inputs the interpreted reference got -- the same generated cparam.local
and, where the case starts from a given state, the same restart file
data/proc00/var.dat -- and must write the state the reference wrote
(data/proc000/var0001.dat; FP64 to 1e-12, FP32 at FP32 rounding), print the
same diagnostics line (run.f90:62) and, where switched on, the same vel01.dat
and qpress01.dat fields (to 1e-11)."""
import os
import struct
import subprocess

import numpy as np
import pytest

from oracle import refbin_parity as rb
from oracle.refsrc import cparam_for
from trapbec_gb300 import abi
from tests.test_refsrc_golden import ARRAYS, CASES, case_params, printed_output_line, reference_state, start_psi

pytestmark = pytest.mark.gpu

DRIVER = os.path.join(os.path.dirname(abi.LIB_PATH), "trapbec_run")
SINGLE = sorted(n for n, r in CASES.items() if r["nprocs"] == 1)


def _field(path, fp64, n):
    rec = rb._read_records(path)[0]
    nx, ny, nz = n
    return np.frombuffer(rec[8:], dtype=np.float64 if fp64 else np.float32).reshape((3, nx, ny, nz))


@pytest.mark.parametrize("name", SINGLE)
def test_driver_reproduces_reference_program_run(name, tmp_path):
    rec = CASES[name]
    p = case_params(rec)
    fp64 = p.precision == abi.FP64
    steps = rec["steps"]
    (tmp_path / "cparam.local").write_text(cparam_for(p, steps, steps, rec["cparam_overrides"]))
    data = tmp_path / "data"
    os.makedirs(data / "proc000", exist_ok=True)
    psi0 = start_psi(name, rec)
    if psi0 is not None:
        rb.write_restart(str(data), psi0.astype(np.complex128 if fp64 else np.complex64), 1, fp64)
    env = dict(os.environ, TRAPBEC_PRECISION="1" if fp64 else "0")
    r = subprocess.run([DRIVER, "cparam.local", "data"], cwd=tmp_path, capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    n = (p.nx, p.ny, p.nz)
    psi, t = rb.gather(str(data), 1, n, 1, fp64)
    got, ref = reference_state(name, psi.astype(np.complex128))
    err = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
    assert err < (1e-12 if fp64 else 2e-6), (name, err)
    assert t == pytest.approx(rec["t"], rel=1e-6 if not fp64 else 1e-14)
    # the output line itime/shots, t, maxPsi, minPsi, meanPsi, intPsi2 (run.f90:62)
    rows = [ln.split() for ln in r.stdout.splitlines()]
    rows = [[float(x) for x in row] for row in rows if len(row) == 6 and row[0].isdigit()]
    want = printed_output_line(rec)
    got = rows[-1][1:]
    # t, maxPsi, minPsi, then meanPsi and intPsi2, which the shipped FP32 build sums
    # sequentially in FP32 (this library's sums are compensated)
    tols = [1e-12] * 5 if fp64 else [2e-6, 2e-6, 2e-6, 1e-5, 1e-5]
    for a, b, tol in zip(got, want, tols):
        assert abs(a - b) <= tol * max(abs(b), want[1]), (name, got, want)
    if rec.get("imag_file"):
        # the imag_var####.dat the imaginary loop wrote after its last step (output.f90:55-62)
        _, _, blk = rb.read_var(str(data / "proc000" / ("imag_var%04d.dat" % rec["imag_steps"])), n, fp64)
        want = ARRAYS[f"{name}__psi_imag"]
        assert float(np.max(np.abs(blk - want)) / np.max(np.abs(want))) < 1e-12
    if rec.get("diag"):
        for f, kind in (("vel01.dat", "vel"), ("qpress01.dat", "qpress")):
            got_f = _field(str(data / "proc000" / f), fp64, n)
            ref_f = ARRAYS[f"{name}__{kind}"]
            assert float(np.max(np.abs(got_f - ref_f)) / np.max(np.abs(ref_f))) < 1e-11
