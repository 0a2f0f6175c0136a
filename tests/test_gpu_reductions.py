"""Precision of the FP32 contexts' compensated reductions.

An FP32 context forms the per-cell terms of its sums in FP32 and adds them
as float-float pairs (TwoSum per thread, float-float trees over the CTA, FP64
over the CTAs).  To see the summation alone, the state here has values whose
per-cell terms are exact in FP32: (kx + i ky)/64 with |kx|, |ky| <= 31, so
|psi|^2 and |psi|^4 are exact products.  The raw sums of trapbec_diag over
256^3 cells (intpsi2 and the quartic sum, no cell volume) must then match the
exact sums to 1e-12 relative, through the tiled and the per-cell diagnostics
kernels; an FP32 running sum would be off by ~1e-3."""
import numpy as np
import pytest

from trapbec_gb300 import Solver, abi
from tests.helpers import params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", [0, 1])
def test_fp32_sums_of_exact_terms_at_256_cubed(kernel):
    n = 256
    p = params(n=(n, n, n), L=(64.0, 64.0, 64.0), prec=abi.FP32, pot="zero")
    rng = np.random.default_rng(11)
    kx = rng.integers(-31, 32, size=n ** 3).astype(np.int64)
    ky = rng.integers(-31, 32, size=n ** 3).astype(np.int64)
    psi = ((kx + 1j * ky) / 64.0).astype(np.complex64).reshape(n, n, n)
    a2 = kx * kx + ky * ky                          # 4096 |psi|^2, exact integers
    intpsi2 = float(int(a2.sum())) / 4096.0
    quartic = float(int((a2 * a2).sum())) / 4096.0 ** 2
    s = Solver(p)
    s.set_kernel(kernel)
    s.set_psi(psi)
    d = s.diag()
    assert abs(d["intpsi2"] / intpsi2 - 1) <= 1e-12, (d["intpsi2"], intpsi2)
    assert abs(d["interaction"] / quartic - 1) <= 1e-12, (d["interaction"], quartic)
    assert d["potential"] == 0.0
    mean_abs = float(np.mean(np.sqrt(a2.astype(np.float64)) / 64.0))
    assert abs(d["meanpsi"] / mean_abs - 1) <= 1e-6     # |psi| itself is rounded to FP32 per cell
    s.close()
