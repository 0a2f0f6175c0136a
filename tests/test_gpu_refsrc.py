"""The CUDA path against golden vectors of the reference's own source.

The fixtures (tests/golden/refsrc_cases.{json,npz}) are the states the
reference's `program run` wrote when its Fortran source was executed by
oracle/fortran_subset.py; see tests/test_refsrc_golden.py.  Here the GPU runs
the same cases through the C ABI: FP64 to 1e-12 relative in psi and the
diagnostics (the CUDA kernels contract to FMA and order the stencil sums
symmetrically, so not bit for bit), FP32 at FP32 rounding, in both real-time
forms the bench uses (three stages and the psi difference); and this
library's file writers against the bytes of the files the reference wrote
(tests/golden/refsrc_files.npz)."""
import os
import struct

import numpy as np
import pytest

from trapbec_gb300 import Solver, abi
from tests.test_refsrc_golden import (ARRAYS, CASES, STEP_CASES, INIT_CASES, case_params, printed_output_line,
                                      reference_state, start_psi)

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("form", [abi.RK3_THREE_STAGE, abi.RK3_PSI_DIFF])
@pytest.mark.parametrize("name", STEP_CASES)
def test_gpu_time_stepping_matches_reference_source(name, form):
    rec = CASES[name]
    p = case_params(rec)
    s = Solver(p)
    s.set_stage_form(form)
    s.set_psi(start_psi(name, rec))
    s.step_rt(rec["steps"])
    got, ref = reference_state(name, s.get_psi().astype(np.complex128))
    ref = ref.astype(np.complex128)
    if p.precision == abi.FP64:
        assert _rel(got, ref) < FP64_TOL, (name, _rel(got, ref))
    else:
        assert _l2(got, ref) < 2e-6, (name, _l2(got, ref))
    t, mx, mn, mean, intpsi2 = printed_output_line(rec)
    d = s.diag()
    tol = FP64_TOL if p.precision == abi.FP64 else 2e-6
    assert abs(d["maxpsi"] - mx) <= tol * mx
    assert abs(d["meanpsi"] - mean) <= tol * mean
    assert abs(d["intpsi2"] - intpsi2) <= (FP64_TOL if p.precision == abi.FP64 else 1e-5) * intpsi2
    assert s.t == pytest.approx(t, rel=1e-6 if p.precision == abi.FP32 else 1e-15)
    s.close()


@pytest.mark.parametrize("name", INIT_CASES)
def test_gpu_initial_states_match_reference_source(name):
    rec = CASES[name]
    s = Solver(case_params(rec))
    s.init_state(rec["init"])
    if "helper" in rec:
        s.init_state(rec["helper"])
    s.step_rt(rec["steps"])   # dt = 0 for the initial states: the reference wrote them after one step
    ref = ARRAYS[f"{name}__psi"]
    tol = 1e-13 if ref.dtype == np.complex128 else 2e-6
    assert _rel(s.get_psi(), ref) < tol, (name, _rel(s.get_psi(), ref))
    s.close()


@pytest.mark.parametrize("name", [n for n, r in CASES.items() if "imag_steps" in r])
def test_gpu_imaginary_time_euler_matches_reference_source(name):
    rec = CASES[name]
    s = Solver(case_params(rec))
    s.init_state("single_vortex")
    if rec["cparam_overrides"].get("phase_imprint_on") == ".true.":
        for _ in range(rec["imag_steps"]):   # run.f90:21-26: Euler step, Psi_norm, phase_imprint
            steps, ratio = s.step_imag(1, abi.IMAG_REF_EULER)
            s.init_state("phase_imprint")
        assert _rel(s.get_psi(), ARRAYS[f"{name}__psi_imag"]) < FP64_TOL
    else:
        steps, ratio = s.step_imag(rec["imag_steps"], abi.IMAG_REF_EULER)
        assert steps == rec["imag_steps"]
    rows = [ln.split() for ln in rec["stdout"]]
    ratios = [float(r[1]) for r in rows if len(r) == 2 and r[0].isdigit()]
    assert ratio == pytest.approx(ratios[-1], rel=1e-12)
    s.step_rt(rec["steps"])
    assert _rel(s.get_psi(), ARRAYS[f"{name}__psi"]) < FP64_TOL
    s.close()


@pytest.mark.parametrize("name", [n for n, r in CASES.items() if r.get("diag")])
def test_gpu_output_diagnostics_match_reference_source(name):
    rec = CASES[name]
    s = Solver(case_params(rec))
    s.set_psi(ARRAYS[f"{name}__psi0"])
    s.step_rt(rec["steps"])
    for kind, got in (("vel", s.velocity()), ("qpress", s.qpressure())):
        ref = ARRAYS[f"{name}__{kind}"]
        assert _rel(got, ref) < 1e-11, (name, kind, _rel(got, ref))
    s.close()


FILES = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "refsrc_files.npz"))


def _records(data):
    out, off = [], 0
    while off < len(data):
        n = struct.unpack("<i", data[off:off + 4])[0]
        out.append((n, data[off + 4:off + 4 + n], struct.unpack("<i", data[off + 4 + n:off + 8 + n])[0]))
        off += 8 + n
    return out


@pytest.mark.parametrize("name", sorted({k.split("__")[0] for k in FILES.files}))
def test_writers_match_reference_files(name, tmp_path):
    """var0001.dat and var.dat written through the C ABI for the state the
    reference wrote are its bytes exactly (src/output.f90:64-75,102-108); the
    vel01.dat / qpress01.dat records have its layout, and values to 1e-11."""
    rec = CASES[name]
    p = case_params(rec)
    s = Solver(p)
    s.set_psi(ARRAYS[f"{name}__psi"])
    s.set_scalar(abi.SCALAR_T, rec["t"])
    s.t = rec["t"]
    steps = rec["steps"]
    d = str(tmp_path)
    os.makedirs(os.path.join(d, "proc000"), exist_ok=True)
    s.write_var(d, itime=steps, shots=steps)
    s.write_restart(d, itime=steps)
    for f in ("var0001.dat", "var.dat"):
        want = FILES[f"{name}__{f}"].tobytes()
        got = open(os.path.join(d, "proc000", f), "rb").read()
        assert got == want, (name, f, len(got), len(want))
    for f, which in (("vel01.dat", abi.FIELD_VELOCITY), ("qpress01.dat", abi.FIELD_QPRESSURE)):
        key = f"{name}__{f}"
        if key not in FILES.files:
            continue
        s.write_field(d, itime=steps, shots=steps, which=which)
        want = _records(FILES[key].tobytes())
        got = _records(open(os.path.join(d, "proc000", f), "rb").read())
        assert len(got) == len(want) == 1
        assert got[0][0] == want[0][0] and got[0][2] == want[0][2] and got[0][1][:8] == want[0][1][:8]
        dt = np.float64 if p.precision == abi.FP64 else np.float32
        a, b = np.frombuffer(got[0][1][8:], dtype=dt), np.frombuffer(want[0][1][8:], dtype=dt)
        assert float(np.max(np.abs(a - b)) / np.max(np.abs(b))) < 1e-11
    s.close()
