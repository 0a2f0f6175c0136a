"""CPU oracle of the warm-start surrogate (test infrastructure only).

A float64 PyTorch-on-CPU restatement of the network in
trapbec_gb300/surrogate.py: the same flat parameter layout (per layer
w[27][Cout][Cin] then b[Cout], in LAYERS order, then the head's wh[16], bh),
the same channels-last tensors, 3x3x3 zero-padded convolutions with
tap = (kd*3 + kh)*3 + kw at offsets -1..1, 2x2x2 mean pooling,
nearest-neighbour upsampling, additive skips before the leaky ReLU and the
linear head added to the Thomas-Fermi base.  Gradients come from autograd in
float64; tests check them against central finite differences and the GPU
kernels against them.  The surrogate has no counterpart in the reference.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

from trapbec_gb300.surrogate import LAYERS, NFEAT, SLOPE, n_params


def conv3(x: torch.Tensor, w: torch.Tensor, b: torch.Tensor | None = None) -> torch.Tensor:
    """x [B,D,H,W,Cin], w [27,Cout,Cin] -> [B,D,H,W,Cout]."""
    cout, cin = w.shape[1], w.shape[2]
    k = w.reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)   # [Cout, Cin, kd, kh, kw]
    y = F.conv3d(x.permute(0, 4, 1, 2, 3), k, bias=b, padding=1)
    return y.permute(0, 2, 3, 4, 1)


def pool2(x):
    B, D, H, W, C = x.shape
    return x.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).mean(dim=(2, 4, 6))


def up2(x):
    return x.repeat_interleave(2, dim=1).repeat_interleave(2, dim=2).repeat_interleave(2, dim=3)


def act(x):
    return F.leaky_relu(x, SLOPE)


def unpack(p: torch.Tensor) -> dict:
    out, off = {}, 0
    for name, ci, co in LAYERS:
        out[name] = (p[off:off + 27 * ci * co].reshape(27, co, ci), p[off + 27 * ci * co:off + 27 * ci * co + co])
        off += 27 * ci * co + co
    out["head"] = (p[off:off + NFEAT], p[off + NFEAT:off + NFEAT + 1])
    assert off + NFEAT + 1 == n_params()
    return out


def _round_bf16(t: torch.Tensor) -> torch.Tensor:
    """Forward: round to BF16 (nearest even); backward: pass the gradient."""
    return t + (t.to(torch.bfloat16).to(t.dtype) - t).detach()


def _grad_to_bf16(t: torch.Tensor) -> torch.Tensor:
    """Identity whose gradient is rounded to BF16."""
    if t.requires_grad:
        t.register_hook(lambda g: g.to(torch.bfloat16).to(g.dtype))
    return t


def forward(p: torch.Tensor, x: torch.Tensor, base: torch.Tensor, bf16: bool = False, keep: dict | None = None):
    """bf16 = True rounds where the GPU path stores BF16: every activation
    and pooled tensor in the forward pass, and the gradient reaching each
    convolution's output (its dz); skip and pooling gradients stay unrounded."""
    P = unpack(p)
    rf = _round_bf16 if bf16 else (lambda t: t)
    rg = _grad_to_bf16 if bf16 else (lambda t: t)

    def c(n, t, skip=None):
        z = rg(conv3(t, *P[n]))
        if skip is not None:
            z = z + skip
        y = rf(act(z))
        if keep is not None:   # activations (and, after backward, their gradients) by layer name
            y.retain_grad()
            keep[n] = y
        return y

    pool = lambda t: rf(pool2(t))
    e0 = c("e0b", c("e0a", x))
    e1 = c("e1b", c("e1a", pool(e0)))
    e2 = c("e2b", c("e2a", pool(e1)))
    e3 = c("e3c", c("e3b", c("e3a", pool(e2))))
    d2 = c("d2b", c("d2a", up2(e3), e2))
    d1 = c("d1b", c("d1a", up2(d2), e1))
    d0 = c("d0b", c("d0a", up2(d1), e0))
    wh, bh = P["head"]
    return base + d0 @ wh + bh


def loss_and_grad(p: np.ndarray, x: np.ndarray, base: np.ndarray, target: np.ndarray, bf16: bool = False,
                  keep: dict | None = None):
    """Loss mean((amp - target)^2) and its gradient w.r.t. the flat parameters
    (float64); `keep` receives each layer's output tensor (with .grad)."""
    pt = torch.tensor(p, dtype=torch.float64, requires_grad=True)
    amp = forward(pt, torch.tensor(x, dtype=torch.float64), torch.tensor(base, dtype=torch.float64), bf16, keep)
    loss = ((amp - torch.tensor(target, dtype=torch.float64)) ** 2).mean()
    loss.backward()
    return float(loss.detach()), pt.grad.numpy().copy()
