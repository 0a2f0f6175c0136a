"""The run.f90-style driver program (trapbec_gb300/lib/trapbec_run)."""
import os
import struct
import subprocess

import numpy as np
import pytest

from trapbec_gb300 import abi

DRIVER = os.path.join(os.path.dirname(abi.LIB_PATH), "trapbec_run")

CPARAM = """! test case in the syntax of cparam.local
real :: Lx=8., Ly=8., Lz=8.
integer, parameter :: Nx=16, Ny=16, Nz=16
complex :: dt=0.01
integer, parameter :: shots=10
integer, parameter :: nsteps={nsteps}
character(len=*), parameter :: boundaries='zero'
character(len=*), parameter :: init_cond='single_vortex'
character(len=*), parameter :: potential='harmonic'
real, parameter :: harm_wx=4, harm_wy=5, harm_wz=6
real, parameter :: omega_z=0.2
logical, parameter :: imaginary_time=.false.
"""


def _run(tmp_path, text, env=None):
    (tmp_path / "cparam.local").write_text(text)
    e = dict(os.environ)
    if env:
        e.update(env)
    return subprocess.run([DRIVER, "cparam.local", "data"], cwd=tmp_path, capture_output=True, text=True, env=e,
                          timeout=300)


def test_driver_parse_error_writes_error_file(tmp_path):
    r = _run(tmp_path, "real :: Lx=8.\ncharacter(len=*), parameter :: boundaries='sticky'\n")
    assert r.returncode == 1
    assert "FATAL ERROR" in r.stdout
    assert "wrong boundaries" in (tmp_path / "ERROR").read_text()


def test_driver_without_device_stops_cleanly(tmp_path, has_gpu):
    if has_gpu:
        pytest.skip("a GPU is present")
    r = _run(tmp_path, CPARAM.format(nsteps=30))
    assert r.returncode == 1
    assert (tmp_path / "ERROR").exists()
    assert (tmp_path / "data" / "dims.log").exists()


def _read_var(path, cdtype, shape):
    data = open(path, "rb").read()
    n = abs(struct.unpack("<i", data[:4])[0])
    rec = data[4:4 + n]
    rs = 8 if cdtype == np.complex128 else 4
    return np.frombuffer(rec[8 + 4 * rs:], dtype=cdtype).reshape(shape), struct.unpack("<4f" if rs == 4 else "<4d",
                                                                                          rec[8:8 + 4 * rs])


@pytest.mark.gpu
def test_driver_run_restart_matches_api(tmp_path):
    from trapbec_gb300 import Solver, parse_cparam
    r = _run(tmp_path, CPARAM.format(nsteps=30))
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if len(l.split()) == 6]
    assert [int(l.split()[0]) for l in lines] == [1, 2, 3]
    psi30, hdr = _read_var(tmp_path / "data" / "proc000" / "var0003.dat", np.complex64, (16, 16, 16))
    assert abs(hdr[3] - 0.30) < 1e-5
    # the same 30 steps through the Python API
    p = parse_cparam(CPARAM.format(nsteps=30))
    p.precision = abi.FP32
    s = Solver(p)
    s.init_state("single_vortex")
    s.step_rt(30)
    assert np.array_equal(s.get_psi(), psi30)
    # restart: nsteps=50 continues from var.dat (itime+1 = 31) to step 50
    r2 = _run(tmp_path, CPARAM.format(nsteps=50))
    assert r2.returncode == 0, r2.stdout + r2.stderr
    assert "restart" in r2.stdout
    psi50, hdr50 = _read_var(tmp_path / "data" / "proc000" / "var0005.dat", np.complex64, (16, 16, 16))
    s.step_rt(20)
    assert np.array_equal(s.get_psi(), psi50)
    timing = (tmp_path / "data" / "timing.log").read_text().split()
    assert int(timing[0]) == 16 ** 3 and float(timing[2]) > 0


@pytest.mark.gpu
def test_driver_vel_and_qpress_files(tmp_path):
    """vel_print / qpress_print: vel##.dat and qpress##.dat after each block
    (run.f90:64-66, output.f90:80-91), equal to the API's fields."""
    from trapbec_gb300 import Solver, parse_cparam
    text = CPARAM.format(nsteps=20) + "logical, parameter :: vel_print=.true.\nlogical, parameter :: qpress_print=.true.\n"
    r = _run(tmp_path, text)
    assert r.returncode == 0, r.stdout + r.stderr
    p = parse_cparam(text)
    p.precision = abi.FP32
    s = Solver(p)
    s.init_state("single_vortex")
    s.step_rt(20)
    for name, want in (("vel02.dat", s.velocity()), ("qpress02.dat", s.qpressure())):
        raw = (tmp_path / "data" / "proc000" / name).read_bytes()
        n = struct.unpack("<i", raw[:4])[0]
        assert n == 8 + 4 * want.size and struct.unpack("<i", raw[-4:])[0] == n
        assert struct.unpack("<2i", raw[4:12]) == (0, 0)
        got = np.frombuffer(raw[12:12 + 4 * want.size], dtype=np.float32).reshape(want.shape)
        assert np.array_equal(got, want)


@pytest.mark.gpu
def test_driver_forcing_helpers_and_slice(tmp_path):
    """forcing every force_freq steps after the output (run.f90:69-74), the
    add_ring / add_dipole helpers at the start (run.f90:37-40) and the
    2D_slice##.log output, replayed through the API."""
    from trapbec_gb300 import Solver, parse_cparam
    text = (CPARAM.format(nsteps=20) + "logical, parameter :: forcing=.true.\ninteger, parameter :: force_freq=5\n"
            "logical, parameter :: add_ring=.true.\nlogical, parameter :: add_dipole=.true.\n"
            "logical, parameter :: gnuplot_2D_print=.true.\n")
    r = _run(tmp_path, text, env={"TRAPBEC_FORCE_SEED": "42"})
    assert r.returncode == 0, r.stdout + r.stderr
    p = parse_cparam(text)
    p.precision = abi.FP32
    s = Solver(p)
    s.init_state("single_vortex")
    s.init_state("add_ring")
    s.init_state("add_dipole")
    for blk in range(1, 5):
        s.step_rt(5)
        if blk == 4:
            break
        s.force_random_points(seed=42, draw=blk)
    psi20, _ = _read_var(tmp_path / "data" / "proc000" / "var0002.dat", np.complex64, (16, 16, 16))
    assert np.array_equal(s.get_psi(), psi20)
    rows = [l.split() for l in (tmp_path / "data" / "proc000" / "2D_slice02.log").read_text().splitlines()]
    vals = np.array([[float(v) for v in row] for row in rows if row])
    assert vals.shape == (16 * 16, 3)
    want = np.abs(psi20[:, :, 0].reshape(-1)) ** 2
    assert np.allclose(vals[:, 2], want, rtol=1e-6, atol=1e-12)
