"""trapbec_psi_stats_noalloc: the Psi_norm / Psi_info statistics computed with
no allocation, checked against trapbec_diag.

This entry point serves callers that cannot let a library allocate device
memory (hosts that pre-reserve the GPU's memory in their own pool and must not
have memory taken behind the pool's back or their streams stalled by an
allocation).  The test hands it a psi that lives in device memory the test
owns, calls it twice in a row through the C ABI, and compares each result with
what trapbec_diag reports for the same state.  The file sorts last so a run
that stops at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from trapbec_gb300 import Solver, abi
from tests.helpers import params, smooth_state

pytestmark = pytest.mark.gpu


def _device_copy(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).reshape(-1).copy()).cuda()


@pytest.mark.parametrize("prec,tol", [(abi.FP64, 1e-12), (abi.FP32, 2e-6)])
def test_noalloc_stats_match_diag_on_two_calls(prec, tol):
    """Two calls in a row, each checked against trapbec_diag of the same state.
    Around the second call (the first has loaded the library's device code and
    looked up the scratch address) neither the device's free memory nor the
    memory torch holds may change: the entry point allocates nothing."""
    torch = pytest.importorskip("torch")
    lib = abi.load()
    p = params(n=(40, 36, 48), L=(10.0, 9.0, 12.0), prec=prec, pot="harmonic", harm=(5.0, 6.0, 7.0))
    s = Solver(p)
    states = [smooth_state(p, seed=31, amp=1.3), smooth_state(p, seed=32, amp=0.7)]
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    dev_states = []
    refs = []
    for psi in states:
        s.set_psi(psi)
        refs.append(s.diag())
        dev_states.append(_device_copy(torch, s.get_psi()))
    s.close()
    torch.cuda.synchronize()
    for call, (dev_psi, ref) in enumerate(zip(dev_states, refs)):
        if call == 1:
            free0 = torch.cuda.mem_get_info()[0]
            held0 = torch.cuda.memory_allocated()
        rc = lib.trapbec_psi_stats_noalloc(C.c_void_p(dev_psi.data_ptr()), dev_psi.numel(), prec,
                                           C.c_void_p(out.data_ptr()), None)
        assert rc == 0, lib.trapbec_last_error()
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free0
            assert torch.cuda.memory_allocated() == held0
        got = out.cpu().numpy()
        for v, k in zip(got, ("intpsi2", "maxpsi", "minpsi", "meanpsi")):
            assert abs(v - ref[k]) <= tol * abs(ref[k]), (call, k, v, ref[k])
