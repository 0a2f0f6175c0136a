"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Tolerances: FP64 results must match the oracle to 1e-12 relative (psi, norm,
energy) after N steps; the kernels reorder the stencil sums and use fused
multiply-adds, so bitwise equality is not expected.  FP32 results are
compared with the FP32 oracle at FP32 rounding levels and their drift
against FP64 is reported by the benchmark.
"""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from trapbec_gb300 import Solver, abi, units
from trapbec_gb300.abi import InitArgs
from tests.helpers import params, smooth_state, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _init_args(init):
    a = InitArgs()
    a.seed = int(init.get("seed", 0))
    a.amp = float(init.get("amp", 1.0))
    for i, v in enumerate(init.get("r_tf2", (0, 0, 0))):
        a.r_tf2[i] = v
    a.ring_radius = float(init.get("ring_radius", 0.0))
    a.core2 = float(init.get("core2", 0.0))
    a.noise_amp = float(init.get("noise_amp", 0.0))
    return a


def _solver_init(s, init):
    s.init_state(init["name"], seed=init.get("seed", 0), amp=init.get("amp", 1.0), r_tf2=init.get("r_tf2", (0, 0, 0)),
                 ring_radius=init.get("ring_radius", 0.0), core2=init.get("core2", 0.0),
                 noise_amp=init.get("noise_amp", 0.0))


@pytest.mark.parametrize("nproc", [(1, 1), (2, 2)])
def test_vortex_line_64_fp64_200_steps(nproc):
    """64^3 FP64 vortex line, 200 RK3 steps: psi, norm and energy to 1e-12."""
    prob, init = units.vortex_line_64(abi.FP64, nproc=nproc)
    p = prob.to_params()
    s = Solver(p)
    _solver_init(s, init)
    o = Oracle(p)
    o.init_state(init["name"], _init_args(init))
    assert rel_err(s.get_psi(), o.get_psi()) < 1e-14
    o.set_psi(s.get_psi())
    d0 = o.diag()
    s.step_rt(init["steps"])
    o.step_rt(init["steps"])
    a, b = s.get_psi(), o.get_psi()
    assert rel_err(a, b) < FP64_TOL
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < FP64_TOL
    dg, do = s.diag(), o.diag()
    for k in ("norm", "energy", "mu", "intpsi2", "maxpsi", "meanpsi"):
        assert abs(dg[k] - do[k]) <= FP64_TOL * abs(do[k]), (k, dg[k], do[k])
    assert abs(s.t - o.t) < 1e-14
    # the run itself conserves norm and energy to RK3 accuracy
    assert abs(do["norm"] / d0["norm"] - 1) < 1e-6


RHS_CASES = [
    dict(bc=abi.BC_ZERO, pot="harmonic", omega=0.3),
    dict(bc=abi.BC_SOLID, pot="harmonic", omega=0.3),
    dict(bc=abi.BC_PERIODIC, pot="zero"),
    dict(bc=abi.BC_ZERO, pot="zero", periodicz=1, vx=0.2),
    dict(bc=abi.BC_SOLID, pot="barrier"),
    dict(bc=abi.BC_ZERO, pot="quartic", harm=(900.0, 8.0, 6.0)),
    dict(bc=abi.BC_ZERO, pot="sphere"),
    dict(bc=abi.BC_ZERO, pot="harmonic_ring", harm=(50.0, 0, 0)),
    dict(bc=abi.BC_ZERO, pot="box_trap"),
    dict(bc=abi.BC_ZERO, pot="channel"),
    dict(bc=abi.BC_ZERO, pot="harmonic", lbeam=1, harm=(3.0, 4.0, 5.0)),
    dict(bc=abi.BC_PERIODIC, pot="zero", two_dim=1),
]


@pytest.mark.parametrize("case", RHS_CASES, ids=lambda c: "-".join(f"{k}{v}" for k, v in c.items()))
def test_get_rhs_parity(case):
    case = dict(case)
    harm = case.pop("harm", (4.0, 5.0, 6.0))
    n = (16, 14, 1 if case.get("two_dim") else 12)
    p = params(n=n, L=(80.0, 70.0, 1.0 if case.get("two_dim") else 60.0), harm=harm, **case)
    psi = smooth_state(p, seed=11)
    s = Solver(p)
    s.set_psi(psi)
    o = Oracle(p)
    o.set_psi(psi)
    assert rel_err(s.get_rhs(), o.get_rhs()) < 1e-13


def test_array_and_mobius_potential():
    p = params(n=(16, 16, 16), L=(60.0, 60.0, 20.0), pot="array", omega=0.1)
    rng = np.random.default_rng(0)
    trap = rng.uniform(0, 2, size=(16, 16, 16))
    psi = smooth_state(p, seed=3)
    for kind in ("array", "mobius"):
        p.potential = abi.POTENTIALS[kind]
        s, o = Solver(p), Oracle(p)
        s.set_trap(trap)
        o.set_trap(trap)
        s.set_psi(psi)
        o.set_psi(psi)
        assert rel_err(s.get_rhs(), o.get_rhs()) < 1e-13
        s.step_rt(3)
        o.step_rt(3)
        assert rel_err(s.get_psi(), o.get_psi()) < FP64_TOL


def test_time_dependent_potential_and_damping():
    """'barrier' depends on t; gamma > 0 damps dt once (run.f90:42)."""
    p = params(n=(16, 16, 12), L=(40.0, 40.0, 30.0), pot="barrier", gamma=0.01, dt=0.02)
    psi = smooth_state(p, seed=8)
    s, o = Solver(p), Oracle(p)
    s.set_psi(psi)
    o.set_psi(psi)
    o.apply_damping()
    s.step_rt(15)
    o.step_rt(15)
    assert rel_err(s.get_psi(), o.get_psi()) < FP64_TOL
    assert abs(s.t - o.t) < 1e-14


@pytest.mark.slow
def test_vortex_ring_256_fp64_parity():
    """The 256^3 vortex-ring workload (TF background x ring of radius 8 in
    z = 0, 1e-3 phase noise, trap (0.05, 0.05, 0.1), g = 1, dt = 0.005) in
    FP64: 60 RK3 steps on the GPU against the oracle from the same state, psi,
    norm and energy to 1e-12 relative."""
    prob, init = units.vortex_ring_256(abi.FP64)
    p = prob.to_params()
    s = Solver(p)
    _solver_init(s, init)
    psi0 = s.get_psi()
    o = Oracle(p)
    o.set_psi(psi0)
    steps = 60
    s.step_rt(steps)
    o.step_rt(steps)
    a, b = s.get_psi(), o.get_psi()
    assert rel_err(a, b) < FP64_TOL
    assert np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()) < FP64_TOL
    dg, do = s.diag(), o.diag()
    for k in ("norm", "energy", "mu", "intpsi2", "maxpsi", "meanpsi"):
        assert abs(dg[k] - do[k]) <= FP64_TOL * abs(do[k]), (k, dg[k], do[k])
    s.close()


def test_fp32_against_fp32_oracle():
    prob, init = units.vortex_line_64(abi.FP32)
    p = prob.to_params()
    p.nx = p.ny = p.nz = 32
    p.lx = p.ly = p.lz = p.lx / 2
    s = Solver(p)
    _solver_init(s, init)
    o = Oracle(p)
    o.set_psi(s.get_psi())
    s.step_rt(20)
    o.step_rt(20)
    a, b = s.get_psi().astype(np.complex128), o.get_psi().astype(np.complex128)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-6
    dg, do = s.diag(), o.diag()
    assert abs(dg["norm"] / do["norm"] - 1) < 1e-6
    assert abs(dg["energy"] / do["energy"] - 1) < 1e-5


def test_fp32_diag_energy_of_fp32_values_matches_fp64():
    """The diagnostics of an FP32 context form the kinetic sum with the stencil
    in difference form, so on a finely resolved state (the 256^3 rotating-trap
    cloud relaxed in imaginary time, h = 0.48 healing lengths) the energy and
    chemical potential of FP32 values match those the FP64 context reports
    for the same values to 1e-6 (measured: 6e-8, the FP32 rounding of the
    cell volume, and 2e-9 for mu), through the tiled and the per-cell kernels."""
    from trapbec_gb300 import reports
    psi, *_ = reports.quench_ground_state(256, max_steps=300)
    out = {}
    for prec, kernel in ((abi.FP64, None), (abi.FP32, None), (abi.FP32, 1)):
        prob, _ = units.rotating_quench_512(prec, n=256)
        s = Solver(prob.to_params())
        if kernel is not None:
            s.set_kernel(kernel)
        s.set_psi(psi if prec == abi.FP32 else psi.astype(np.complex128))
        out[(prec, kernel)] = s.diag()
        s.close()
    ref = out[(abi.FP64, None)]
    for key in ((abi.FP32, None), (abi.FP32, 1)):
        d = out[key]
        assert abs(d["energy"] / ref["energy"] - 1) < 1e-6, (key, d["energy"], ref["energy"])
        assert abs(d["mu"] / ref["mu"] - 1) < 1e-6, (key, d["mu"], ref["mu"])
        # sum |psi|^2 without the cell volume (an FP32 context forms h in FP32, as
        # the reference's FP32 build does, so dV differs by ~1e-7)
        assert abs(d["intpsi2"] / ref["intpsi2"] - 1) < 1e-8, (key, d["intpsi2"], ref["intpsi2"])


def test_imag_euler_matches_reference_loop():
    p = params(n=(16, 16, 16), L=(8.0, 8.0, 8.0), pot="harmonic", harm=(6.0, 6.0, 6.0), dt=0.005)
    psi = smooth_state(p, seed=9)
    s, o = Solver(p), Oracle(p)
    s.set_psi(psi)
    o.set_psi(psi)
    sd, ratio = s.step_imag(7, abi.IMAG_REF_EULER)
    r_o = o.step_imag_euler(7)
    assert sd == 7
    assert rel_err(s.get_psi(), o.get_psi()) < FP64_TOL
    assert abs(ratio - r_o) < 1e-12 * abs(r_o)


def test_imag_rk3_renorm_matches_oracle():
    p = params(n=(20, 20, 20), L=(10.0, 10.0, 10.0), pot="harmonic", harm=(100.0, 120.0, 90.0), dt=0.01,
               omega=0.2)
    psi = smooth_state(p, seed=12)
    s, o = Solver(p), Oracle(p)
    s.set_psi(psi)
    o.set_psi(psi)
    sg, rg = s.step_imag(150, abi.IMAG_RK3_RENORM, 0.0)      # fixed number of steps
    so, ro = o.step_imag_rk3(150, 0.0)
    assert sg == so == 150
    assert rel_err(s.get_psi(), o.get_psi()) < 1e-11
    dg, do = s.diag(), o.diag()
    assert abs(dg["energy"] - do["energy"]) < 1e-12 * abs(do["energy"])
    assert abs(dg["norm"] - do["norm"]) < 1e-12 * do["norm"]
    # now to convergence: same stopping step (or one apart at the threshold)
    sg2, rg2 = s.step_imag(5000, abi.IMAG_RK3_RENORM, 1e-10)
    so2, ro2 = o.step_imag_rk3(5000, 1e-10)
    assert abs(sg2 - so2) <= 1 and rg2 <= 1e-10 and ro2 <= 1e-10
    assert rel_err(s.get_psi(), o.get_psi()) < 1e-8


def test_imag_rk3_absolute_stop_matches_oracle():
    """The absolute stop |E_n - E_{n-1}| * scale < tol (the workload's |dE| <
    tol with the energy in the caller's unit): the same stopping step as the
    oracle's loop (one apart at the threshold); stat_out is |dE| * scale."""
    p = params(n=(20, 20, 20), L=(10.0, 10.0, 10.0), pot="harmonic", harm=(100.0, 120.0, 90.0), dt=0.01,
               omega=0.2)
    psi = smooth_state(p, seed=13)
    scale, tol = 37.5, 3e-9
    s, o = Solver(p), Oracle(p)
    s.set_psi(psi)
    o.set_psi(psi)
    s.set_imag_stop(abi.STOP_ABS, scale)
    o.set_imag_stop(abi.STOP_ABS, scale)
    sg, rg = s.step_imag(5000, abi.IMAG_RK3_RENORM, tol)
    so, ro = o.step_imag_rk3(5000, tol)
    assert 10 < sg < 5000 and abs(sg - so) <= 1, (sg, so)
    assert rg < tol and ro < tol
    assert rel_err(s.get_psi(), o.get_psi()) < 1e-8
    # the energy per unit norm: |dE| / N0 * scale < tol
    s2, o2 = Solver(p), Oracle(p)
    s2.set_psi(psi)
    o2.set_psi(psi)
    s2.set_imag_stop(abi.STOP_ABS_PER_NORM, scale)
    o2.set_imag_stop(abi.STOP_ABS_PER_NORM, scale)
    sn, rn = s2.step_imag(5000, abi.IMAG_RK3_RENORM, tol)
    on, ron = o2.step_imag_rk3(5000, tol)
    assert 10 < sn < 5000 and abs(sn - on) <= 1, (sn, on)
    assert rn < tol and ron < tol
    # back to the relative test: from the converged state it stops within a few steps
    s.set_imag_stop(abi.STOP_REL)
    sg2, rg2 = s.step_imag(100, abi.IMAG_RK3_RENORM, 1e-6)
    assert sg2 <= 3 and rg2 <= 1e-6
    with pytest.raises(abi.TrapbecError):
        s.set_imag_stop(abi.STOP_ABS, -1.0)


def test_imag_rk3_split_calls_report_the_same_last_change():
    """A relaxation split over two calls ends on the same |dE|/|E| as one call
    over the same steps: the energy of a call's final state comes from the same
    stage-1 evaluation as every other energy the loop compares."""
    p = params(n=(20, 20, 20), L=(10.0, 10.0, 10.0), pot="harmonic", harm=(100.0, 120.0, 90.0), dt=0.01,
               omega=0.2)
    psi = smooth_state(p, seed=14)
    one, two = Solver(p), Solver(p)
    one.set_psi(psi)
    two.set_psi(psi)
    n1, r1 = one.step_imag(100, abi.IMAG_RK3_RENORM, 0.0)
    na, ra = two.step_imag(60, abi.IMAG_RK3_RENORM, 0.0)
    nb, rb = two.step_imag(40, abi.IMAG_RK3_RENORM, 0.0)
    assert n1 == 100 and na == 60 and nb == 40
    assert rel_err(one.get_psi(), two.get_psi()) < 1e-13
    assert abs(rb - r1) <= 1e-3 * r1, (rb, r1)


INIT_STATES = ["constant", "thomas_fermi", "soliton", "single_vortex", "sausage", "crow", "random_points",
               "leap_frog", "vortex_rings", "lattice", "lattice2", "bundle", "line_of_lines", "linked_rings",
               "random_phase"]


@pytest.mark.parametrize("helper,pot", [("add_noise", "harmonic"), ("add_ring", "harmonic"),
                                        ("add_dipole", "harmonic"), ("phase_imprint", "harmonic"),
                                        ("add_pcurrent", "barrier"), ("add_pcurrent", "channel"),
                                        ("add_pcurrent", "harmonic_ring")])
def test_state_helpers(helper, pot):
    """Helpers act on the current state (initial.f90:669-870)."""
    p = params(n=(24, 24, 16), L=(60.0, 60.0, 30.0), harm=(3.0, 4.0, 5.0), pot=pot)
    p.winding_number = 3
    p.ring_rad = 6.0
    s, o = Solver(p), Oracle(p)
    a = InitArgs()
    a.seed = 5
    s.init_state("thomas_fermi")
    o.init_state("thomas_fermi", a)
    s.init_state(helper, seed=5)
    o.init_state(helper, a)
    assert rel_err(s.get_psi(), o.get_psi()) < 1e-13


@pytest.mark.parametrize("name", INIT_STATES)
def test_initial_states(name):
    p = params(n=(24, 24, 16), L=(40.0, 40.0, 30.0), harm=(3.0, 4.0, 5.0))
    p.winding_number = 2
    p.vor_ring_count = 2
    p.ring_rad = 6.0
    s, o = Solver(p), Oracle(p)
    a = InitArgs()
    a.seed = 77
    s.init_state(name, seed=77)
    o.init_state(name, a)
    assert rel_err(s.get_psi(), o.get_psi()) < 1e-13


@pytest.mark.parametrize("name", ["tf_vortex_line", "tf_vortex_ring", "tf_noise"])
def test_workload_states(name):
    p = params(n=(24, 24, 20), L=(40.0, 40.0, 30.0))
    init = dict(name=name, amp=1.3, r_tf2=(1 / 150.0, 1 / 140.0, 1 / 90.0), core2=2.5, ring_radius=6.0,
                noise_amp=1e-2, seed=5)
    s, o = Solver(p), Oracle(p)
    _solver_init(s, init)
    o.init_state(name, _init_args(init))
    assert rel_err(s.get_psi(), o.get_psi()) < 1e-13


def test_ghosted_layout_roundtrip():
    p = params(n=(10, 12, 8), L=(5.0, 6.0, 4.0), bc=abi.BC_SOLID, periodicz=1)
    psi = smooth_state(p, seed=6)
    s, o = Solver(p), Oracle(p)
    o.set_psi(psi)
    g = o.get_psi_ghosted()
    s.set_psi(g, abi.LAYOUT_GHOSTED)
    assert np.array_equal(s.get_psi(), psi)
    gs = s.get_psi(abi.LAYOUT_GHOSTED)
    # faces as ghost_comm leaves them; edges/corners are never written (zero)
    m = np.zeros(g.shape, bool)
    m[3:-3, 3:-3, :] = True
    m[3:-3, :, 3:-3] = True
    m[:, 3:-3, 3:-3] = True
    assert np.array_equal(gs[m], g[m])


def test_launch_count_and_timing():
    p = params(n=(16, 16, 16), L=(8.0, 8.0, 8.0), pot="harmonic", harm=(3.0, 3.0, 3.0))
    s = Solver(p)
    s.set_psi(smooth_state(p, seed=1))
    n0 = s.launch_count()
    s.step_rt(4)
    assert s.launch_count() - n0 == 12  # three fused stage kernels per RK3 step
    assert s.last_kernel_ms() > 0


def _read_fortran_record(f):
    import struct
    out = b""
    while True:
        (lead,) = struct.unpack("<i", f.read(4))
        n = abs(lead)
        out += f.read(n)
        f.read(4)
        if lead >= 0:
            return out


def test_var_and_restart_files(tmp_path):
    """var####.dat follows output.f90:75-78 and bin/gather.m:13-28; var.dat has
    the 3 records of output.f90:103-108; reading it back restores psi."""
    import struct
    for prec in (abi.FP32, abi.FP64):
        p = params(n=(8, 10, 6), L=(4.0, 5.0, 3.0), prec=prec)
        s = Solver(p)
        psi = smooth_state(p, seed=2).astype(s.cdtype)
        s.set_psi(psi)
        s.set_scalar(abi.SCALAR_T, 1.25)
        d = str(tmp_path / f"data{prec}")
        s.write_var(d, itime=200, shots=100)
        rs = 8 if prec == abi.FP64 else 4
        with open(f"{d}/proc000/var0002.dat", "rb") as f:
            rec = _read_fortran_record(f)
        cx, cy = struct.unpack("<2i", rec[:8])
        fmt = "<4d" if rs == 8 else "<4f"
        Lx, Ly, Lz, t = struct.unpack(fmt, rec[8:8 + 4 * rs])
        arr = np.frombuffer(rec[8 + 4 * rs:], dtype=s.cdtype).reshape(8, 10, 6)
        assert (cx, cy) == (0, 0) and (Lx, Ly, Lz) == (4.0, 5.0, 3.0) and t == 1.25
        assert np.array_equal(arr, psi)
        s.write_restart(d, itime=300)
        with open(f"{d}/proc000/var.dat", "rb") as f:
            r1, r2, r3 = (_read_fortran_record(f) for _ in range(3))
        assert struct.unpack("<i", r1)[0] == 301 and len(r2) == rs
        s2 = Solver(p)
        nstart = s2.read_restart(d)
        assert nstart == 301 and s2.t == 1.25
        assert np.array_equal(s2.get_psi(), psi)


DIAG_CASES = [(abi.FP64, abi.BC_ZERO, 0, (1, 1)), (abi.FP64, abi.BC_ZERO, 0, (2, 2)),
              (abi.FP64, abi.BC_PERIODIC, 0, (1, 2)), (abi.FP64, abi.BC_SOLID, 1, (2, 1)),
              (abi.FP32, abi.BC_ZERO, 0, (1, 1)), (abi.FP32, abi.BC_PERIODIC, 0, (2, 2))]


@pytest.mark.parametrize("prec,bc,pz,nproc", DIAG_CASES)
def test_velocity_and_qpressure(prec, bc, pz, nproc):
    """get_phase velocity and get_qpressure (diagnostic.f90:27-84), after a few
    RK3 steps, against the oracle: FP64 to 1e-12 of the field's maximum,
    FP32 to 2e-5 (atan2/hypot of the two libraries differ by an ulp or two;
    a vortex-free smooth state keeps the phase away from the branch cut's
    sign ambiguity)."""
    p = params(n=(24, 32, 20), L=(6.0, 8.0, 5.0), prec=prec, bc=bc, periodicz=pz, nproc=nproc, omega=0.2)
    rng = np.random.default_rng(17)
    psi = smooth_state(p, seed=9) + 0.02 * (rng.normal(size=(24, 32, 20)) + 1j * rng.normal(size=(24, 32, 20)))
    s = Solver(p)
    s.set_psi(psi)
    s.step_rt(3)
    o = Oracle(p)
    o.set_psi(s.get_psi())
    tol = FP64_TOL if prec == abi.FP64 else 2e-5
    for got, want in ((s.velocity(), o.velocity()), (s.qpressure(), o.qpressure())):
        assert got.shape == (3, 24, 32, 20)
        assert np.all(np.isfinite(got))
        err = np.abs(got.astype(np.float64) - want.astype(np.float64))
        assert err.max() <= tol * np.abs(want).max(), err.max()


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_forcing_random_points(prec):
    """force_random_points (force.f90:12-54): the draws lie in
    [-Lx/4, Lx/4] x [-Ly/4, Ly/4] with dir = +-1, are reproducible per
    (seed, draw) and differ between draws; the forced state matches the
    oracle's force_vortex at the drawn point."""
    p = params(n=(32, 24, 16), L=(16.0, 12.0, 8.0), prec=prec, nproc=(2, 2))
    psi = smooth_state(p, seed=3) + 0.3
    s = Solver(p)
    s.set_psi(psi)
    o = Oracle(p)
    o.set_psi(s.get_psi())
    seen = set()
    for draw in range(6):
        x0, y0, d = s.force_random_points(seed=7, draw=draw)
        assert -4.0 <= x0 <= 4.0 and -3.0 <= y0 <= 3.0 and d in (-1.0, 1.0)
        seen.add((x0, y0))
        o.force_vortex(x0, y0, d)
    assert len(seen) == 6
    s2 = Solver(p)
    assert s2.force_random_points(seed=7, draw=3) == Solver.force_random_points(s2, seed=7, draw=3)
    tol = FP64_TOL if prec == abi.FP64 else 1e-5   # six FP32 multiplications by sin/cos/atan2 values
    assert rel_err(s.get_psi(), o.get_psi()) < tol
