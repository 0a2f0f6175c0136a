"""Pins the surrogate's CPU oracle (no GPU): autograd gradients against
central finite differences, and the tap / layout convention of conv3."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import nn_oracle
from trapbec_gb300.surrogate import LAYERS, NFEAT, n_params


def _problem(S=8, B=1, seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(n_params())
    off = 0
    for _, ci, co in LAYERS:
        p[off:off + 27 * ci * co] = rng.normal(0, np.sqrt(2.0 / (27 * ci)), 27 * ci * co)
        p[off + 27 * ci * co:off + 27 * ci * co + co] = rng.normal(0, 0.05, co)
        off += 27 * ci * co + co
    p[off:off + NFEAT + 1] = rng.normal(0, 0.3, NFEAT + 1)
    x = rng.normal(size=(B, S, S, S, 16))
    base = rng.uniform(0, 1, size=(B, S, S, S))
    tgt = rng.uniform(0, 1, size=(B, S, S, S))
    return p, x, base, tgt


def test_conv3_tap_convention():
    """tap (kd, kh, kw) reads x[d + kd - 1, h + kh - 1, w + kw - 1], zero outside."""
    rng = np.random.default_rng(1)
    x = torch.tensor(rng.normal(size=(1, 4, 5, 6, 2)))
    w = torch.zeros(27, 2, 2, dtype=torch.float64)
    tap = (2 * 3 + 1) * 3 + 0
    w[tap, 1, 0] = 1.0
    y = nn_oracle.conv3(x, w)
    want = torch.zeros(1, 4, 5, 6, dtype=torch.float64)
    want[:, :3, :, 1:] = x[:, 1:, :, :5, 0]
    assert torch.equal(y[..., 1], want)
    assert torch.count_nonzero(y[..., 0]) == 0


def test_oracle_gradient_matches_finite_differences():
    p, x, base, tgt = _problem()
    loss, g = nn_oracle.loss_and_grad(p, x, base, tgt)
    rng = np.random.default_rng(7)
    # coordinates spread over every layer's weights and biases and the head
    idx, off = [], 0
    for _, ci, co in LAYERS:
        idx += list(rng.integers(off, off + 27 * ci * co, 2)) + [off + 27 * ci * co]
        off += 27 * ci * co + co
    idx += [off, off + NFEAT]
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (nn_oracle.loss_and_grad(pp, x, base, tgt)[0] - nn_oracle.loss_and_grad(pm, x, base, tgt)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-7 * np.abs(g).max(), (i, fd, g[i])
