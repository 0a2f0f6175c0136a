"""The Fortran-subset interpreter (oracle/fortran_subset.py) on small programs
of its own: the semantics it claims -- kinds and promotion, one rounding per
operation in source order, component-wise complex x real, integer division and
powers, sequential SUM, array sections with lower bounds, SELECT CASE on
strings, the emulated MPI of a 2 x 2 process grid, unformatted records --
checked against numpy evaluations of the same expressions."""
import struct

import numpy as np
import pytest

from oracle import fortran_subset as fs


def run_src(tmp_path, text, nprocs=1, real_kind=4, includes=None):
    path = tmp_path / "prog.f90"
    path.write_text(text)
    inc = {"mpif.h": fs.MPIF_H}
    inc.update(includes or {})
    return fs.run(str(tmp_path), ["prog.f90"], inc, nprocs, real_kind, str(tmp_path))


def out_values(rank):
    return [ln.split() for ln in rank.stdout]


def test_scalar_semantics_single_precision(tmp_path):
    src = """
module m
  implicit none
  real :: a=0.1, b=3.
  complex :: z=(0.3,-1.7)
  integer :: n=7
end module
program p
  use m
  implicit none
  real :: r
  complex :: c
  r = a*b + a/b
  print*, r
  c = z*z + 2*z
  print*, real(c), aimag(c)
  print*, n/2, (-n)/2, mod(-n,3), 2**10
  r = abs(z)
  print*, r
  c = z/4.
  print*, real(c), aimag(c)
end program
"""
    r = run_src(tmp_path, src)[0]
    v = out_values(r)
    f = np.float32
    a, b = f(0.1), f(3.0)
    assert float(v[0][0]) == float(a * b + a / b)
    zr, zi = f(0.3), f(-1.7)
    re_ = (zr * zr - zi * zi) + f(2) * zr
    im_ = (zr * zi + zi * zr) + f(2) * zi
    assert float(v[1][0]) == float(re_) and float(v[1][1]) == float(im_)
    assert [int(x) for x in v[2]] == [3, -3, -1, 1024]
    assert float(v[3][0]) == float(np.float32(np.hypot(np.float64(zr), np.float64(zi))))
    assert float(v[4][0]) == float(zr / f(4)) and float(v[4][1]) == float(zi / f(4))


def test_double_build_and_sequential_sum(tmp_path):
    src = """
program p
  implicit none
  real, allocatable :: x(:)
  integer :: i
  allocate(x(-2:5))
  do i=-2,5
    x(i) = 1./(i+3.5)
  end do
  print*, sum(x(0:5)), maxval(x), x(-2)
end program
"""
    r = run_src(tmp_path, src, real_kind=8)[0]
    v = [float(t) for t in out_values(r)[0]]
    xs = [1.0 / (i + 3.5) for i in range(-2, 6)]
    acc = 0.0
    for q in xs[2:]:
        acc += q
    assert v[0] == acc and v[1] == max(xs) and v[2] == xs[0]


def test_select_case_strings_and_control_flow(tmp_path):
    src = """
module m
  character(len=*), parameter :: pot='harmonic'
end module
program p
  use m
  implicit none
  integer :: i, s
  s = 0
  select case(pot)
    case('zero','box')
      s = 1
    case('harmonic')
      s = 2
    case default
      s = 3
  end select
  do i=1,10,3
    if (i==4) then
      s = s + 100
    else if (i>5) then
      s = s + 10
    else
      s = s + 1
    end if
  end do
  print*, s, i
end program
"""
    r = run_src(tmp_path, src)[0]
    assert out_values(r)[0] == ["123", "13"]


def test_emulated_mpi_grid(tmp_path):
    """ISEND/IRECV/WAIT around a periodic 2 x 2 Cartesian grid, REDUCE and BCAST."""
    src = """
module m
  implicit none
  include 'mpif.h'
  integer :: rank, nprocs, ierror, comm2d, left, right, req(2), stat(MPI_STATUS_SIZE)
  integer :: dims(2)=0, coords(2)
  logical :: per(2)=.true.
  real :: sbuf(3), rbuf(3), tot
end module
program p
  use m
  implicit none
  call MPI_INIT(ierror)
  call MPI_COMM_SIZE(MPI_COMM_WORLD, nprocs, ierror)
  call MPI_COMM_RANK(MPI_COMM_WORLD, rank, ierror)
  call MPI_DIMS_CREATE(nprocs,2,dims,ierror)
  call MPI_CART_CREATE(MPI_COMM_WORLD,2,dims,per,.true.,comm2D,ierror)
  call MPI_CART_COORDS(comm2D, rank, 2, coords, ierror)
  call MPI_CART_SHIFT(comm2D,0,1,left,right,ierror)
  sbuf = rank + 0.5
  call MPI_ISEND(sbuf,3,MPI_REAL,left,7,comm2D,req(1),ierror)
  call MPI_IRECV(rbuf,3,MPI_REAL,right,7,comm2D,req(2),ierror)
  call MPI_WAIT(req(1),stat,ierror) ; call MPI_WAIT(req(2),stat,ierror)
  call MPI_REDUCE(rbuf(1),tot,1,MPI_REAL,MPI_SUM,0,comm2d,ierror)
  call MPI_BCAST(tot, 1, MPI_REAL, 0,comm2d,ierror)
  print*, rank, coords(1), coords(2), left, right, rbuf(2), tot
  call MPI_FINALIZE(ierror)
end program
"""
    ranks = run_src(tmp_path, src, nprocs=4)
    rows = [[float(x) for x in out_values(r)[0]] for r in ranks]
    for r, row in enumerate(rows):
        cx, cy = r // 2, r % 2
        right = ((cx + 1) % 2) * 2 + cy
        assert row[:5] == [r, cx, cy, ((cx - 1) % 2) * 2 + cy, right]
        assert row[5] == right + 0.5          # received from the right neighbour
        assert row[6] == 0.5 + 1.5 + 2.5 + 3.5


def test_unformatted_records_round_trip(tmp_path):
    (tmp_path / "d").mkdir()
    src = """
program p
  implicit none
  complex :: z(2,3)
  integer :: it, i, j
  real :: t
  do i=1,2
    do j=1,3
      z(i,j) = cmplx(i, 10*j)
    end do
  end do
  open(unit=98,file='./d/f.dat',form='unformatted',status='replace')
  write(98) 42
  write(98) 1.5
  write(98) z(1:2,2:3)
  close(98)
  open(unit=98,file='./d/f.dat',form='unformatted')
  read(98) it
  read(98) t
  close(98)
  print*, it, t
end program
"""
    r = run_src(tmp_path, src)[0]
    assert out_values(r)[0] == ["42", "1.5"]
    data = open(tmp_path / "d" / "f.dat", "rb").read()
    n = struct.unpack("<i", data[:4])[0]
    assert n == 4 and struct.unpack("<i", data[4:8])[0] == 42
    third = data[12 + 12:]   # after the records of 42 and 1.5 (4-byte markers around 4-byte payloads)
    m = struct.unpack("<i", third[:4])[0]
    vals = np.frombuffer(third[4:4 + m], dtype=np.complex64)
    # column-major z(1:2,2:3): z(1,2), z(2,2), z(1,3), z(2,3)
    assert vals.tolist() == [1 + 20j, 2 + 20j, 1 + 30j, 2 + 30j]


def test_unsupported_constructs_raise(tmp_path):
    with pytest.raises(fs.FortranError):
        run_src(tmp_path, "program p\n  implicit none\n  goto 10\nend program\n")
