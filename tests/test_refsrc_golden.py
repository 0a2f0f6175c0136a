"""The oracle against golden vectors of the reference's own source.

tests/golden/refsrc_cases.{json,npz} hold the states that `program run`
(src/run.f90) and the modules it uses produced when executed statement by
statement by oracle/fortran_subset.py (generator:
tests/golden/make_refsrc_fixtures.py): the RK3 time stepping on 1 rank and
on a 2 x 2 process grid in the FP64 build and the shipped FP32 one, every
boundary type, the rotating and advective frames, the potential library and
the laser, imaginary-time Euler, the init_cond library and the helpers of
run.f90:37-40, and the output-time diagnostics.  The oracle restates the same
statements in C++ with the same evaluation order, so it must reproduce them
bit for bit (initial states, which go through libm's transcendental
functions, to 1e-14)."""
import json
import os
import platform

import numpy as np
import pytest

from oracle.pyoracle import Oracle
from trapbec_gb300.abi import default_params

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def load_cases():
    meta = json.load(open(os.path.join(GOLD, "refsrc_cases.json")))
    arrays = np.load(os.path.join(GOLD, "refsrc_cases.npz"))
    return meta, arrays


META, ARRAYS = load_cases()
CASES = META["cases"]
# The interpreter took ABS of a complex (hypot) and the other intrinsic
# functions from the generating machine's libm, as the oracle takes them from
# this one's: where the two libms are the same the oracle must agree bit for
# bit; another libm (aarch64 glibc's hypot rounds differently in the last
# place) leaves ulp-level differences.
SAME_LIBM = (META.get("platform", {}).get("machine") == platform.machine() and
             META.get("platform", {}).get("libc") == " ".join(platform.libc_ver()))


def case_params(rec):
    p = default_params()
    for k, v in rec["params"].items():
        setattr(p, k, v)
    return p


def start_psi(name, rec):
    """The state a case started from: kept in the fixtures, or (for the cases
    at the workload's own size) the workload's start state rebuilt."""
    if f"{name}__psi0" in ARRAYS.files:
        return ARRAYS[f"{name}__psi0"]
    if rec.get("start") == "tf_vortex_line":
        from oracle import refbin_parity as rb
        from trapbec_gb300 import units
        prob, init = units.vortex_line_64(1)
        return rb.start_state(prob.to_params(), init)
    return None


def reference_state(name, got):
    """(got, want) restricted to the cells the fixture kept."""
    if f"{name}__idx" in ARRAYS.files:
        return got.ravel()[ARRAYS[f"{name}__idx"]], ARRAYS[f"{name}__psi_sample"]
    return got, ARRAYS[f"{name}__psi"]


def printed_output_line(rec):
    """The run.f90:62 line `itime/shots, t, maxPsi, minPsi, meanPsi, intPsi2` of the last output."""
    rows = [ln.split() for ln in rec["stdout"]]
    rows = [r for r in rows if len(r) == 6 and r[0].isdigit()]
    return [float(x) for x in rows[-1][1:]]


def oracle_run(name, rec):
    """The oracle taken through the same steps as the reference case `name`."""
    p = case_params(rec)
    o = Oracle(p)
    psi0 = start_psi(name, rec)
    ratio = None
    if "init" in rec:
        o.init_state(rec["init"])
        if "helper" in rec:
            o.init_state(rec["helper"])
        o.step_rt(rec["steps"])
    elif "imag_steps" in rec:
        o.init_state("single_vortex")
        if rec["cparam_overrides"].get("phase_imprint_on") == ".true.":
            for _ in range(rec["imag_steps"]):   # run.f90:21-26: Euler step, Psi_norm, phase_imprint
                ratio = o.step_imag_euler(1)
                o.init_state("phase_imprint")
        else:
            ratio = o.step_imag_euler(rec["imag_steps"])
        o.step_rt(rec["steps"])
    else:
        o.set_psi(psi0)
        if p.gamma != 0.0:
            o.apply_damping()
        o.step_rt(rec["steps"])
    return o, ratio


STEP_CASES = [n for n, r in CASES.items() if "init" not in r and "imag_steps" not in r]
INIT_CASES = [n for n, r in CASES.items() if "init" in r]


def test_fixture_set_is_complete():
    names = set(CASES)
    for must in ("line16_np1_fp64", "line16_np4_fp64", "line16_np1_fp32", "line16_np4_fp32", "rot_np4_fp64",
                 "solid_pz_np4_fp64", "periodic_np4_fp64", "advective_fp64", "imag_euler_fp64",
                 "diag_np4_fp64", "init_lattice2_fp64", "helper_add_ring_fp64"):
        assert must in names, must


@pytest.mark.parametrize("name", STEP_CASES)
def test_oracle_reproduces_reference_time_stepping_bitwise(name):
    rec = CASES[name]
    o, _ = oracle_run(name, rec)
    got, ref = reference_state(name, o.get_psi())
    got = got.astype(ref.dtype)
    if SAME_LIBM:
        assert np.array_equal(got.view(np.uint8), ref.view(np.uint8)), \
            (name, float(np.max(np.abs(got - ref))))
    else:
        err = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
        assert err < (1e-15 if ref.dtype == np.complex128 else 1e-6), (name, err)
    assert o.t == pytest.approx(rec["t"], rel=1e-6 if ref.dtype == np.complex64 else 1e-15)


@pytest.mark.parametrize("name", STEP_CASES)
def test_oracle_diagnostics_match_reference_output_line(name):
    """Psi_info / Psi_norm as the reference printed them after the last step."""
    rec = CASES[name]
    o, _ = oracle_run(name, rec)
    t, mx, mn, mean, intpsi2 = printed_output_line(rec)
    d = o.diag()
    fp32 = rec["params"]["precision"] == 0
    tol = 2e-6 if fp32 else 1e-13
    assert abs(d["maxpsi"] - mx) <= tol * mx
    assert abs(d["minpsi"] - mn) <= tol * max(mx, 1e-30)
    assert abs(d["meanpsi"] - mean) <= tol * mean
    assert abs(d["intpsi2"] - intpsi2) <= (1e-5 if fp32 else 1e-13) * intpsi2


@pytest.mark.parametrize("name", INIT_CASES)
def test_oracle_reproduces_reference_initial_states(name):
    """Cases that start from the reference's init_cond (the library of initial
    states and helpers with dt = 0; the 'mobius' potential, whose Trap
    mesh_init builds only then, with two steps)."""
    rec = CASES[name]
    o, _ = oracle_run(name, rec)
    ref = ARRAYS[f"{name}__psi"]
    got = o.get_psi()
    err = float(np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300))
    assert err < (1e-14 if ref.dtype == np.complex128 else 1e-6), (name, err)


@pytest.mark.parametrize("name", [n for n, r in CASES.items() if "imag_steps" in r])
def test_oracle_reproduces_reference_imaginary_time_euler(name):
    rec = CASES[name]
    o, ratio = oracle_run(name, rec)
    ref = ARRAYS[f"{name}__psi"]
    err = float(np.max(np.abs(o.get_psi() - ref)) / np.max(np.abs(ref)))
    assert err < 1e-14
    # run.f90:28 prints itime/shots and imag_Psiratio after every imaginary step
    rows = [ln.split() for ln in rec["stdout"]]
    ratios = [float(r[1]) for r in rows if len(r) == 2 and r[0].isdigit()]
    assert len(ratios) == rec["imag_steps"]
    assert ratio == pytest.approx(ratios[-1], rel=1e-14)


@pytest.mark.parametrize("name", [n for n, r in CASES.items() if r.get("diag")])
def test_oracle_diagnostics_fields_match_reference_files(name):
    """get_phase velocity and get_qpressure (vel01.dat, qpress01.dat)."""
    rec = CASES[name]
    p = case_params(rec)
    o, _ = oracle_run(name, rec)
    for kind, got in (("vel", o.velocity()), ("qpress", o.qpressure())):
        ref = ARRAYS[f"{name}__{kind}"]
        err = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
        assert err < 1e-12, (name, kind, err)
    assert p.nprocx * p.nprocy == rec["nprocs"]
