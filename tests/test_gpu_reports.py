"""FP32 against FP64 precision reports on small grids (the full-size runs
are the reports' defaults: the 256^3 ring over 2000 steps, and the 512^3
quench from its imaginary-time ground state, FP32 over the 5000-step ramp
and FP64 over the first 1000 steps)."""
import pytest

from trapbec_gb300 import reports

pytestmark = pytest.mark.gpu


def test_ring_fp32_drift_and_l2():
    r = reports.fp32_vs_fp64(n=64, steps=200, chunk=50)
    # RK3 is not norm-preserving (|P(i lambda dt)| < 1): the FP64 run drifts by
    # the scheme's own amount; FP32 must add less than 1e-6 to it
    assert abs(r["fp64"]["norm_drift"]) < 1e-6
    assert abs(r["fp32"]["norm_drift"]) < 1e-6
    assert abs(r["fp32_vs_fp64"]["norm_rel"]) < 1e-6
    assert r["fp32_vs_fp64"]["l2_rel_psi"] < 1e-4
    assert len(r["fp32_vs_fp64"]["checkpoints"]) == 4


def test_quench_checkpoints():
    ground = reports.quench_ground_state(64, max_steps=300)
    assert 1 <= ground[1] <= 300
    runs = {g: reports.quench_checkpoints(n=64, steps=100, every=50, chunk=25, fp32_steps=200, gauge=g,
                                          ground=ground) for g in ("state_mu", "tf_mu")}
    r = runs["state_mu"]
    assert [c["step"] for c in r["fp32_vs_fp64"]["checkpoints"]] == [50, 100]
    assert [c["step"] for c in r["fp32"]["checkpoints"]] == [50, 100, 150, 200]
    for c in r["fp32_vs_fp64"]["checkpoints"]:
        assert abs(c["norm_rel"]) < 1e-6 and abs(c["energy_rel"]) < 1e-5
    assert r["fp32_vs_fp64"]["l2_rel_psi"] < 1e-4
    assert abs(r["fp32"]["norm_drift"]) < 1e-6
    # in the Thomas-Fermi unit scale the ground state turns its phase and the
    # FP32 norm grows (the oracle shows the same: test_oracle_fp32_gauge)
    assert runs["tf_mu"]["fp32"]["norm_drift"] > 10 * abs(r["fp32"]["norm_drift"])
