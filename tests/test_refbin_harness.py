"""The reference-binary parity harness (oracle/refbin_parity.py) up to the
compiler call, with no Fortran compiler or MPI: the cparam.local it writes
parses back to the same parameters, the per-rank restart files hold the
three records the reference's reader expects and reassemble to the start
state, the output gather places every rank's block by its recorded coords,
and the FP64 source patch touches only the MPI datatypes.  The run against
the reference binary itself skips where mpif90 / mpiexec are missing."""
import os
import struct

import numpy as np
import pytest

from oracle import refbin_parity as H
from trapbec_gb300 import abi, parse_cparam, units


def test_mpi_dims_create_matches_the_balanced_grids():
    assert H.mpi_dims_create(1) == (1, 1)
    assert H.mpi_dims_create(2) == (2, 1)
    assert H.mpi_dims_create(4) == (2, 2)
    assert H.mpi_dims_create(6) == (3, 2)
    assert H.mpi_dims_create(8) == (4, 2)
    assert H.mpi_dims_create(16) == (4, 4)
    assert [H.rank_coords(r, (2, 2)) for r in range(4)] == [(0, 0), (0, 1), (1, 0), (1, 1)]


@pytest.mark.parametrize("which", ["line", "ring"])
def test_cparam_round_trip(which):
    prob = (units.vortex_line_64(abi.FP64)[0] if which == "line" else units.vortex_ring_256(abi.FP64)[0])
    prob.Omega = 0.003
    p = prob.to_params()
    text = H.cparam_text(p, nsteps=200, shots=50)
    q = parse_cparam(text)
    for k in ("nx", "ny", "nz", "boundaries", "periodicz", "two_dim", "potential", "lbeam", "winding_number",
              "vor_ring_count"):
        assert getattr(q, k) == getattr(p, k), k
    for k in ("lx", "ly", "lz", "dt_re", "dt_im", "gamma", "harm_wx", "harm_wy", "harm_wz", "wbeam",
              "advective_vx", "omega_z", "ring_rad"):
        assert getattr(q, k) == getattr(p, k), k     # repr round-trips a double exactly
    assert q.potential_off > 1e38 and q.t_spindown > 1e38
    # every name run.f90 and its modules read is declared
    for name in ("shots", "nsteps", "init_cond", "imaginary_time", "imag_nsteps", "full_binary_output",
                 "imaginary_output", "gnuplot_2d_print", "qpress_print", "vel_print", "forcing", "force_freq",
                 "add_pcurrent", "add_ring", "add_dipole", "phase_imprint_on", "vor_line_count"):
        assert f"{name}=" in text, name


@pytest.mark.parametrize("nprocs,fp64", [(1, True), (4, True), (4, False)])
def test_restart_files_hold_the_reader_records(tmp_path, nprocs, fp64):
    rng = np.random.default_rng(3)
    n = (8, 6, 5)
    psi = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex128 if fp64 else np.complex64)
    H.write_restart(str(tmp_path), psi, nprocs, fp64, itime=1, t=0.0)
    dims = H.mpi_dims_create(nprocs)
    mx, my = n[0] // dims[0], n[1] // dims[1]
    back = np.zeros_like(psi)
    for r in range(nprocs):
        assert (tmp_path / ("proc%03d" % r)).is_dir()            # the writer's directories exist
        it, t, blk = H.read_restart(str(tmp_path / ("proc%02d" % r) / "var.dat"), (mx, my, n[2]), fp64)
        assert it == 1 and t == 0.0
        cx, cy = H.rank_coords(r, dims)
        back[cx * mx:(cx + 1) * mx, cy * my:(cy + 1) * my] = blk
        # record markers: 4-byte itime, kind-sized t, the whole local block
        raw = open(tmp_path / ("proc%02d" % r) / "var.dat", "rb").read()
        assert struct.unpack("<i", raw[:4])[0] == 4
        assert struct.unpack("<i", raw[12:16])[0] == (8 if fp64 else 4)
    assert np.array_equal(back, psi)


def _write_var_rank(path, coords, L, t, blk, fp64):
    rs = "<4d" if fp64 else "<4f"
    payload = struct.pack("<2i", *coords) + struct.pack(rs, *L, t) + blk.tobytes()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "wb") as f:
        n = struct.pack("<i", len(payload))
        f.write(n + payload + n)


@pytest.mark.parametrize("fp64", [True, False])
def test_gather_places_blocks_by_recorded_coords(tmp_path, fp64):
    rng = np.random.default_rng(4)
    n = (8, 8, 4)
    psi = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex128 if fp64 else np.complex64)
    dims = H.mpi_dims_create(4)
    blocks = H.split_ranks(psi, dims)
    # files written in a shuffled rank order: the gather must use the coords inside each file
    for r in (2, 0, 3, 1):
        _write_var_rank(str(tmp_path / ("proc%03d" % r) / "var0003.dat"), H.rank_coords(r, dims),
                        (10.0, 11.0, 12.0), 0.25, blocks[r], fp64)
    got, t = H.gather(str(tmp_path), 3, n, 4, fp64)
    assert np.array_equal(got, psi)
    assert t == pytest.approx(0.25)


def test_fp64_patch_touches_only_the_mpi_datatypes():
    src = ("call MPI_ISEND(ghost_l1,nmeshz*nmeshy,MPI_COMPLEX,left,tag(1),comm2D,lsend(1),ierror)\n"
           "call MPI_REDUCE(x,y,1,MPI_REAL,MPI_MAX,0,comm2d,ierror)\n"
           "call MPI_REDUCE(a,b,1,MPI_LOGICAL,MPI_LAND,0,comm2d,ierror)\n"
           "real :: MPI_REALITY_CHECK\n")
    out = H.fp64_patch(src)
    assert "MPI_DOUBLE_COMPLEX,left" in out and "1,MPI_DOUBLE_PRECISION,MPI_MAX" in out
    assert "MPI_LOGICAL" in out and "MPI_REALITY_CHECK" in out
    assert "MPI_COMPLEX," not in out


def test_workloads_decompose_evenly():
    for name, prob, init, steps, nprocs in H.workloads():
        dims = H.mpi_dims_create(nprocs)
        assert prob.n[0] % dims[0] == 0 and prob.n[1] % dims[1] == 0, name
        assert tuple(prob.nproc) == dims, name
        assert steps > 0


def test_reference_binary_parity():
    ok, why = H.available()
    if not ok:
        pytest.skip(why)
    ref_src = os.environ.get("TRAPBEC_REFERENCE_SRC")
    if not ref_src or not os.path.isdir(ref_src):
        pytest.skip("TRAPBEC_REFERENCE_SRC does not name the reference's src directory")
    assert H.main(["--ref-src", ref_src, "--only", "vortex_line_64_np4"]) == 0
