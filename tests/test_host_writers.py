"""The host-state writers of the C ABI (trapbec_write_var_host,
trapbec_write_restart_host) against the bytes of the files the reference's
own source wrote (tests/golden/refsrc_files.npz: var0001.dat and var.dat of
`program run`, output.f90:64-75,102-108), for the state the reference wrote.
Host code only: no GPU."""
import ctypes as C
import os

import numpy as np
import pytest

from trapbec_gb300 import abi
from tests.test_refsrc_golden import ARRAYS, CASES, case_params

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = np.load(os.path.join(HERE, "golden", "refsrc_files.npz"))


@pytest.mark.parametrize("name", sorted({k.split("__")[0] for k in FILES.files}))
def test_host_writers_write_the_reference_files(name, tmp_path):
    lib = abi.load()
    rec = CASES[name]
    p = case_params(rec)
    psi = np.ascontiguousarray(ARRAYS[f"{name}__psi"],
                               dtype=np.complex128 if p.precision == abi.FP64 else np.complex64)
    d = str(tmp_path)
    os.makedirs(os.path.join(d, "proc000"))
    steps = rec["steps"]
    assert lib.trapbec_write_var_host(C.byref(p), d.encode(), steps, steps, rec["t"], 0, psi.ctypes.data) == abi.OK
    assert lib.trapbec_write_restart_host(C.byref(p), d.encode(), steps, rec["t"], psi.ctypes.data) == abi.OK
    for f in ("var0001.dat", "var.dat"):
        want = FILES[f"{name}__{f}"].tobytes()
        got = open(os.path.join(d, "proc000", f), "rb").read()
        assert got == want, (name, f, len(got), len(want))


def test_host_writers_reject_bad_arguments(tmp_path):
    lib = abi.load()
    p = abi.default_params()
    buf = np.zeros(p.nx * p.ny * p.nz, dtype=np.complex128)
    d = str(tmp_path).encode()
    assert lib.trapbec_write_var_host(None, d, 1, 1, 0.0, 0, buf.ctypes.data) == abi.ERR_ARG
    assert lib.trapbec_write_var_host(C.byref(p), d, 1, 0, 0.0, 0, buf.ctypes.data) == abi.ERR_ARG
    assert lib.trapbec_write_var_host(C.byref(p), d, 1, 1, 0.0, 0, None) == abi.ERR_ARG
    assert lib.trapbec_write_restart_host(C.byref(p), None, 1, 0.0, buf.ctypes.data) == abi.ERR_ARG
