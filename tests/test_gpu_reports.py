"""FP32 against FP64 precision reports on small grids (the full-size runs
are the reports' defaults: 256^3 x 2000 steps and 512^3 x 1000 steps)."""
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
    r = reports.quench_checkpoints(n=64, steps=100, every=50, chunk=25)
    assert [c["step"] for c in r["fp32_vs_fp64"]["checkpoints"]] == [50, 100]
    for c in r["fp32_vs_fp64"]["checkpoints"]:
        assert abs(c["norm_rel"]) < 1e-6 and abs(c["energy_rel"]) < 1e-5
    assert r["fp32_vs_fp64"]["l2_rel_psi"] < 1e-4
