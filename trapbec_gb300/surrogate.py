"""Learned warm start for imaginary-time ground states.

A 3D convolutional encoder-decoder (four levels S, S/2, S/4, S/8 with 16,
32, 64, 128 channels, 2x2x2 mean pooling down, nearest-neighbour upsampling
up, additive skips, leaky ReLU, about 1.8M parameters) maps the trap
potential and the instance parameters, as 16 input channels on the grid, to
the ground-state amplitude |psi| in the reference's units, predicted as a
correction to the Thomas-Fermi amplitude sqrt(max(0, 1 - pot)).

All arithmetic runs in the library's kernels (include/trapbec_surrogate.h):
BF16 tensor-core convolutions with FP32 accumulation for the forward pass,
the input gradients and the weight gradients, FP32 head, loss and Adam.
PyTorch only provides device buffers and the stream.

The prediction is used only as the initial guess of the batched
imaginary-time solver; the guess keeps the seeded 1e-2 noise of the
Thomas-Fermi guess so that rotating instances can still break the symmetry
and nucleate vortices.  The phase is not predicted: in the axially symmetric
traps of this workload the ground state is either real (no vortices) or
carries a vortex lattice whose positions break the symmetry, and a smooth
phase field can represent neither.  Relaxation from the Thomas-Fermi guess
stays the fallback and the yardstick: both runs stop on the same relative
energy change, and their final energies are compared.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import abi, units

# (name, Cin, Cout) of the 3x3x3 convolutions, in forward order
LAYERS = [("e0a", 16, 16), ("e0b", 16, 16), ("e1a", 16, 32), ("e1b", 32, 32), ("e2a", 32, 64),
          ("e2b", 64, 64), ("e3a", 64, 128), ("e3b", 128, 128), ("e3c", 128, 128), ("d2a", 128, 64),
          ("d2b", 64, 64), ("d1a", 64, 32), ("d1b", 32, 32), ("d0a", 32, 16), ("d0b", 16, 16)]
NFEAT = 16
SLOPE = 0.05
# The committed weights (weights/surrogate_128.npz, record in
# weights/surrogate_128_train.json) were trained on draws 0..TRAIN_DRAWS-1 of
# units.ground_state_draws(seed=TRAIN_SEED, grids=(128,)); draws from
# TRAIN_DRAWS on are held out.
TRAIN_SEED = 2024
TRAIN_DRAWS = 2000


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the surrogate's kernels need a CUDA device")
    return torch


def n_params() -> int:
    return sum(27 * ci * co + co for _, ci, co in LAYERS) + NFEAT + 1


# ---- inputs -------------------------------------------------------------------

def features(prob: units.TrapProblem) -> tuple[np.ndarray, np.ndarray]:
    """Input channels [S, S, S, 16] (FP32) and the Thomas-Fermi amplitude
    base [S, S, S] of one instance, in the reference's units.

    0: pot (harmonic, finite_diff.f90:33-34, clipped at 2)   1: TF amplitude
    2: log10(g)/3   3: Omega / (0.7 omega_perp)   4: (omega_z/omega_perp - 0.5)/3.5
    5, 6, 7: grid spacings hx', hy', hz' (healing lengths)   8: Omega/mu
    9: log10(mu/omega_perp)/3   10..15: zero."""
    p = prob.to_params()
    n = (p.nx, p.ny, p.nz)
    ax = []
    for m, L in zip(n, (p.lx, p.ly, p.lz)):
        i = np.arange(1, m + 1)
        ax.append(((2 * i - 1) / (2.0 * m) * L - L / 2.0) / L)   # x'/L'
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    pot = p.harm_wx * X ** 2 + p.harm_wy * Y ** 2 + p.harm_wz * Z ** 2
    base = np.sqrt(np.maximum(0.0, 1.0 - pot))
    f = np.zeros(n + (NFEAT,), dtype=np.float32)
    f[..., 0] = np.minimum(pot, 2.0)
    f[..., 1] = base
    f[..., 2:10] = feature_consts(prob)
    return f, base.astype(np.float32)


def feature_consts(prob: units.TrapProblem) -> np.ndarray:
    """Channels 2-9 of `features` (constant over the grid), FP32."""
    p = prob.to_params()
    wp, wz = prob.omega[0], prob.omega[2]
    return np.array([math.log10(prob.g) / 3.0, prob.Omega / (0.7 * wp), (wz / wp - 0.5) / 3.5, p.lx / p.nx,
                     p.ly / p.ny, p.lz / p.nz, prob.Omega / prob.mu, math.log10(prob.mu / wp) / 3.0],
                    dtype=np.float32)


def features_device(lib, prob: units.TrapProblem, x, base, stream=None) -> None:
    """`features(prob)` built on the device: x a [S, S, S, 16] BF16 view, base a
    [S, S, S] FP32 view (CUDA tensors); equal to the host arrays rounded to BF16."""
    p = prob.to_params()
    c = feature_consts(prob)
    rc = lib.tbsg_features(x.data_ptr(), base.data_ptr(), p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, p.harm_wx, p.harm_wy,
                           p.harm_wz, c.ctypes.data, stream)
    if rc:
        raise RuntimeError(f"tbsg_features failed ({rc})")


def stable_dtau(prob: units.TrapProblem, frac: float = 0.6) -> float:
    """A trap-units imaginary step at `frac` of the RK3 stability limit: the
    6th-order Laplacian's largest eigenvalue is (1088/180) sum 1/h'^2 and RK3
    is stable on [-2.51, 0]; dtau = dtau'/(2 mu)."""
    p = prob.to_params()
    lam = (1088.0 / 180.0) * sum((m / L) ** 2 for m, L in ((p.nx, p.lx), (p.ny, p.ly), (p.nz, p.lz)))
    return frac * 2.51 / lam / (2.0 * prob.mu)


# ---- the network ----------------------------------------------------------------

class Surrogate:
    """The encoder-decoder on an S^3 grid (S divisible by 8) for `batch` samples."""

    def __init__(self, S: int, batch: int = 1, seed: int = 0):
        if S % 8:
            raise ValueError("S must be a multiple of 8")
        torch = _torch()
        self.t = torch
        self.lib = abi.load()
        self.S, self.B = S, batch
        self.dev = torch.device("cuda", torch.cuda.current_device())
        # flat FP32 parameters: per layer w [27][Cout][Cin] then b [Cout]; then head wh[16], bh
        self.np = n_params()
        self.p = torch.zeros(self.np, dtype=torch.float32, device=self.dev)
        self.g = torch.zeros_like(self.p)
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.step_t = 0
        self.view = {}
        off = 0
        for name, ci, co in LAYERS:
            self.view[name] = (off, off + 27 * ci * co, ci, co)
            off += 27 * ci * co + co
        self.view["head"] = (off, off + NFEAT, NFEAT, 1)
        rng = np.random.default_rng(seed)
        host = np.zeros(self.np, dtype=np.float32)
        for name, ci, co in LAYERS:
            w0, b0, _, _ = self.view[name]
            host[w0:b0] = rng.normal(0.0, math.sqrt(2.0 / (27 * ci)), 27 * ci * co)
        # the head starts at zero: the untrained network returns the Thomas-Fermi amplitude
        self.p.copy_(torch.from_numpy(host))
        self.wb = {n: torch.empty(27 * ci * co, dtype=torch.bfloat16, device=self.dev) for n, ci, co in LAYERS}
        self.wt = {n: torch.empty(27 * ci * co, dtype=torch.bfloat16, device=self.dev) for n, ci, co in LAYERS}
        self._alloc()
        self.prep()

    # -- buffers ------------------------------------------------------------------
    def _alloc(self):
        t, B = self.t, self.B
        S = [self.S, self.S // 2, self.S // 4, self.S // 8]
        bf = lambda lev, c: t.empty((B, S[lev], S[lev], S[lev], c), dtype=t.bfloat16, device=self.dev)
        f32 = lambda lev, c: t.empty((B, S[lev], S[lev], S[lev], c), dtype=t.float32, device=self.dev)
        A = {}
        A["x0"] = bf(0, 16); A["e0a"] = bf(0, 16); A["e0"] = bf(0, 16)
        A["p1"] = bf(1, 16); A["e1a"] = bf(1, 32); A["e1"] = bf(1, 32)
        A["p2"] = bf(2, 32); A["e2a"] = bf(2, 64); A["e2"] = bf(2, 64)
        A["p3"] = bf(3, 64); A["e3a"] = bf(3, 128); A["e3b"] = bf(3, 128); A["e3"] = bf(3, 128)
        A["u2"] = bf(2, 128); A["d2a"] = bf(2, 64); A["d2"] = bf(2, 64)
        A["u1"] = bf(1, 64); A["d1a"] = bf(1, 32); A["d1"] = bf(1, 32)
        A["u0"] = bf(0, 32); A["d0a"] = bf(0, 16); A["d0"] = bf(0, 16)
        self.A = A
        G = {}
        for name, (lev, c) in {"d0": (0, 16), "d0a": (0, 16), "u0": (0, 32), "e0": (0, 16), "e0a": (0, 16),
                               "d1": (1, 32), "d1a": (1, 32), "u1": (1, 64), "e1": (1, 32), "e1a": (1, 32),
                               "p1": (1, 16), "d2": (2, 64), "d2a": (2, 64), "u2": (2, 128), "e2": (2, 64),
                               "e2a": (2, 64), "p2": (2, 32), "e3": (3, 128), "e3b": (3, 128), "e3a": (3, 128),
                               "p3": (3, 64)}.items():
            G[name] = f32(lev, c)
        self.G = G
        self.dz = {lev: t.empty((B, S[lev], S[lev], S[lev], 16 << lev), dtype=t.bfloat16, device=self.dev)
                   for lev in range(4)}
        # the second dz buffer of a level: an input gradient fused with the activation derivative below
        # reads one and writes the other
        self.dz2 = {lev: t.empty_like(self.dz[lev]) for lev in range(4)}
        sb = max(self.lib.tbsg_conv3_wgrad_scratch_bytes(ci, co, B, S[lv], S[lv], S[lv])
                 for (n, ci, co), lv in zip(LAYERS, [0, 0, 1, 1, 2, 2, 3, 3, 3, 2, 2, 1, 1, 0, 0]))
        self.scratch = t.empty(sb // 4 + 1, dtype=t.float32, device=self.dev)
        self.scratch_bytes = sb
        nvox = B * self.S ** 3
        self.partials = t.empty(self.lib.tbsg_head_partials(nvox, NFEAT), dtype=t.float32, device=self.dev)
        self.head_out = t.empty(NFEAT + 2, dtype=t.float32, device=self.dev)
        self.clip_part = t.empty(1024, dtype=t.float32, device=self.dev)
        self.clip_out = t.zeros(2, dtype=t.float32, device=self.dev)
        self.amp = t.empty((B, self.S, self.S, self.S), dtype=t.float32, device=self.dev)

    # -- plumbing -------------------------------------------------------------------
    def _st(self):
        return C.c_void_p(self.t.cuda.current_stream().cuda_stream)

    @staticmethod
    def _ptr(x):
        return C.c_void_p(x.data_ptr()) if x is not None else None

    def _ck(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: surrogate kernel error {rc}")

    def _pw(self, name):
        w0, b0, ci, co = self.view[name]
        return self.p[w0:b0], self.p[b0:b0 + co]

    def prep(self):
        """FP32 master weights -> BF16 working copies (both layouts)."""
        for name, ci, co in LAYERS:
            w, _ = self._pw(name)
            self._ck(self.lib.tbsg_weight_prep(self._ptr(w), self._ptr(self.wb[name]), self._ptr(self.wt[name]),
                                               ci, co, self._st()), "weight_prep")

    def _conv(self, name, x, y, D, skip=None, act=True):
        _, ci, co = next(l for l in LAYERS if l[0] == name)
        _, b = self._pw(name)
        self._ck(self.lib.tbsg_conv3_fwd(self._ptr(x), ci, self._ptr(self.wb[name]), self._ptr(b), self._ptr(skip),
                                         self._ptr(y), None, 0, co, self.B, D, D, D, 1 if act else 0, SLOPE,
                                         self._st()), f"conv {name}")

    def _conv_bwd(self, name, x_in, dz, D, g_in):
        _, ci, co = next(l for l in LAYERS if l[0] == name)
        w0, b0, _, _ = self.view[name]
        dw, db = self.g[w0:b0], self.g[b0:b0 + co]
        self._ck(self.lib.tbsg_conv3_wgrad(self._ptr(x_in), ci, self._ptr(dz), co, self.B, D, D, D, self._ptr(dw),
                                           self._ptr(db), self._ptr(self.scratch), self.scratch_bytes, self._st()),
                 f"wgrad {name}")
        if g_in is not None:
            self._ck(self.lib.tbsg_conv3_fwd(self._ptr(dz), co, self._ptr(self.wt[name]), None, None, None,
                                             self._ptr(g_in), 0, ci, self.B, D, D, D, 0, 0.0, self._st()),
                     f"dgrad {name}")

    def _conv_bwd_act(self, name, x_in, dz, D, y_in, dz_in, dskip=None):
        """Weight gradient of `name`, then its input gradient fused with the
        activation derivative of the layer below (y_in its output): dz_in and,
        optionally, dskip += the activation's input gradient."""
        _, ci, co = next(l for l in LAYERS if l[0] == name)
        w0, b0, _, _ = self.view[name]
        dw, db = self.g[w0:b0], self.g[b0:b0 + co]
        self._ck(self.lib.tbsg_conv3_wgrad(self._ptr(x_in), ci, self._ptr(dz), co, self.B, D, D, D, self._ptr(dw),
                                           self._ptr(db), self._ptr(self.scratch), self.scratch_bytes, self._st()),
                 f"wgrad {name}")
        self._ck(self.lib.tbsg_conv3_dgrad_act(self._ptr(dz), co, self._ptr(self.wt[name]), self._ptr(y_in),
                                               self._ptr(dz_in), self._ptr(dskip), ci, self.B, D, D, D, SLOPE,
                                               self._st()), f"dgrad_act {name}")

    def _act_bwd(self, g, y, dz, dskip=None):
        self._ck(self.lib.tbsg_act_bwd(self._ptr(g), self._ptr(y), self._ptr(dz), self._ptr(dskip), y.numel(), SLOPE,
                                       self._st()), "act_bwd")

    # -- forward / backward ---------------------------------------------------------------
    def forward(self, x: "torch.Tensor", base: "torch.Tensor") -> "torch.Tensor":
        """x: [B, S, S, S, 16] BF16 (or FP32, converted), base: [B, S, S, S] FP32.
        Returns the predicted amplitude [B, S, S, S] (FP32, a view of an
        internal buffer)."""
        A, S, L = self.A, self.S, self.lib
        st = self._st()
        if x.dtype == self.t.float32:
            self._ck(L.tbsg_f32_to_bf16(self._ptr(x), self._ptr(A["x0"]), x.numel(), st), "to_bf16")
        else:
            A["x0"].copy_(x)
        self.base = base
        s0, s1, s2, s3 = S, S // 2, S // 4, S // 8
        self._conv("e0a", A["x0"], A["e0a"], s0); self._conv("e0b", A["e0a"], A["e0"], s0)
        self._ck(L.tbsg_pool2_fwd(self._ptr(A["e0"]), self._ptr(A["p1"]), 16, self.B, s0, s0, s0, st), "pool")
        self._conv("e1a", A["p1"], A["e1a"], s1); self._conv("e1b", A["e1a"], A["e1"], s1)
        self._ck(L.tbsg_pool2_fwd(self._ptr(A["e1"]), self._ptr(A["p2"]), 32, self.B, s1, s1, s1, st), "pool")
        self._conv("e2a", A["p2"], A["e2a"], s2); self._conv("e2b", A["e2a"], A["e2"], s2)
        self._ck(L.tbsg_pool2_fwd(self._ptr(A["e2"]), self._ptr(A["p3"]), 64, self.B, s2, s2, s2, st), "pool")
        self._conv("e3a", A["p3"], A["e3a"], s3); self._conv("e3b", A["e3a"], A["e3b"], s3)
        self._conv("e3c", A["e3b"], A["e3"], s3)
        self._ck(L.tbsg_up2_fwd(self._ptr(A["e3"]), self._ptr(A["u2"]), 128, self.B, s3, s3, s3, st), "up")
        self._conv("d2a", A["u2"], A["d2a"], s2, skip=A["e2"]); self._conv("d2b", A["d2a"], A["d2"], s2)
        self._ck(L.tbsg_up2_fwd(self._ptr(A["d2"]), self._ptr(A["u1"]), 64, self.B, s2, s2, s2, st), "up")
        self._conv("d1a", A["u1"], A["d1a"], s1, skip=A["e1"]); self._conv("d1b", A["d1a"], A["d1"], s1)
        self._ck(L.tbsg_up2_fwd(self._ptr(A["d1"]), self._ptr(A["u0"]), 32, self.B, s1, s1, s1, st), "up")
        self._conv("d0a", A["u0"], A["d0a"], s0, skip=A["e0"]); self._conv("d0b", A["d0a"], A["d0"], s0)
        h0, h1, _, _ = self.view["head"]
        self._ck(L.tbsg_head_fwd(self._ptr(A["d0"]), NFEAT, self._ptr(self.p[h0:h1]), self._ptr(self.p[h1:h1 + 1]),
                                 self._ptr(base), self._ptr(self.amp), self.amp.numel(), st), "head")
        return self.amp

    def backward(self, target: "torch.Tensor", fused: bool = True) -> "torch.Tensor":
        """Gradients of mean((amp - target)^2) of the last forward() into
        self.g; returns the loss (a 1-element device tensor).  fused: input
        gradients that feed an activation derivative directly are computed
        with it (tbsg_conv3_dgrad_act) instead of through an FP32 gradient
        in memory; the parameter gradients are the same, bit for bit."""
        if fused:
            return self._backward_fused(target)
        A, G, S, L, dz = self.A, self.G, self.S, self.lib, self.dz
        st = self._st()
        s0, s1, s2, s3 = S, S // 2, S // 4, S // 8
        h0, h1, _, _ = self.view["head"]
        self._ck(L.tbsg_head_loss(self._ptr(A["d0"]), NFEAT, self._ptr(self.p[h0:h1]), self._ptr(self.p[h1:h1 + 1]),
                                  self._ptr(self.base), self._ptr(target), self.amp.numel(), self._ptr(G["d0"]),
                                  self._ptr(self.partials), self._ptr(self.head_out), st), "head_loss")
        self.g[h0:h1 + 1].copy_(self.head_out[1:NFEAT + 2])
        for k in ("e0", "e1", "e2"):
            G[k].zero_()
        # level 0 decoder
        self._act_bwd(G["d0"], A["d0"], dz[0]); self._conv_bwd("d0b", A["d0a"], dz[0], s0, G["d0a"])
        self._act_bwd(G["d0a"], A["d0a"], dz[0], G["e0"]); self._conv_bwd("d0a", A["u0"], dz[0], s0, G["u0"])
        self._ck(L.tbsg_up2_bwd(self._ptr(G["u0"]), self._ptr(G["d1"]), 32, self.B, s1, s1, s1, st), "up_bwd")
        # level 1 decoder
        self._act_bwd(G["d1"], A["d1"], dz[1]); self._conv_bwd("d1b", A["d1a"], dz[1], s1, G["d1a"])
        self._act_bwd(G["d1a"], A["d1a"], dz[1], G["e1"]); self._conv_bwd("d1a", A["u1"], dz[1], s1, G["u1"])
        self._ck(L.tbsg_up2_bwd(self._ptr(G["u1"]), self._ptr(G["d2"]), 64, self.B, s2, s2, s2, st), "up_bwd")
        # level 2 decoder
        self._act_bwd(G["d2"], A["d2"], dz[2]); self._conv_bwd("d2b", A["d2a"], dz[2], s2, G["d2a"])
        self._act_bwd(G["d2a"], A["d2a"], dz[2], G["e2"]); self._conv_bwd("d2a", A["u2"], dz[2], s2, G["u2"])
        self._ck(L.tbsg_up2_bwd(self._ptr(G["u2"]), self._ptr(G["e3"]), 128, self.B, s3, s3, s3, st), "up_bwd")
        # bottleneck
        self._act_bwd(G["e3"], A["e3"], dz[3]); self._conv_bwd("e3c", A["e3b"], dz[3], s3, G["e3b"])
        self._act_bwd(G["e3b"], A["e3b"], dz[3]); self._conv_bwd("e3b", A["e3a"], dz[3], s3, G["e3a"])
        self._act_bwd(G["e3a"], A["e3a"], dz[3]); self._conv_bwd("e3a", A["p3"], dz[3], s3, G["p3"])
        self._ck(L.tbsg_pool2_bwd(self._ptr(G["p3"]), self._ptr(G["e2"]), 64, self.B, s2, s2, s2, st), "pool_bwd")
        # encoder
        self._act_bwd(G["e2"], A["e2"], dz[2]); self._conv_bwd("e2b", A["e2a"], dz[2], s2, G["e2a"])
        self._act_bwd(G["e2a"], A["e2a"], dz[2]); self._conv_bwd("e2a", A["p2"], dz[2], s2, G["p2"])
        self._ck(L.tbsg_pool2_bwd(self._ptr(G["p2"]), self._ptr(G["e1"]), 32, self.B, s1, s1, s1, st), "pool_bwd")
        self._act_bwd(G["e1"], A["e1"], dz[1]); self._conv_bwd("e1b", A["e1a"], dz[1], s1, G["e1a"])
        self._act_bwd(G["e1a"], A["e1a"], dz[1]); self._conv_bwd("e1a", A["p1"], dz[1], s1, G["p1"])
        self._ck(L.tbsg_pool2_bwd(self._ptr(G["p1"]), self._ptr(G["e0"]), 16, self.B, s0, s0, s0, st), "pool_bwd")
        self._act_bwd(G["e0"], A["e0"], dz[0]); self._conv_bwd("e0b", A["e0a"], dz[0], s0, G["e0a"])
        self._act_bwd(G["e0a"], A["e0a"], dz[0]); self._conv_bwd("e0a", A["x0"], dz[0], s0, None)
        return self.head_out[0:1]

    def _backward_fused(self, target):
        """backward() with every activation derivative fused into the kernel
        that forms the gradient it multiplies: the head's loss gradient, the
        input gradients of the convolutions above an activation, the pooling
        and the upsampling gradients."""
        A, G, S, L, dz, dz2 = self.A, self.G, self.S, self.lib, self.dz, self.dz2
        st = self._st()
        s0, s1, s2, s3 = S, S // 2, S // 4, S // 8
        h0, h1, _, _ = self.view["head"]
        self._ck(L.tbsg_head_loss_act(self._ptr(A["d0"]), self._ptr(self.p[h0:h1]), self._ptr(self.p[h1:h1 + 1]),
                                      self._ptr(self.base), self._ptr(target), self.amp.numel(), self._ptr(dz[0]),
                                      SLOPE, self._ptr(self.partials), self._ptr(self.head_out), st), "head_loss_act")
        self.g[h0:h1 + 1].copy_(self.head_out[1:NFEAT + 2])
        for k in ("e0", "e1", "e2"):
            G[k].zero_()
        # decoder: level 0, 1, 2 (the skip gradients accumulate into e0, e1, e2)
        for lev, D, (b, a_), up, ynext, cn in ((0, s0, ("d0b", "d0a"), "u0", "d1", 32),
                                               (1, s1, ("d1b", "d1a"), "u1", "d2", 64),
                                               (2, s2, ("d2b", "d2a"), "u2", "e3", 128)):
            self._conv_bwd_act(b, A[a_], dz[lev], D, A[a_], dz2[lev], G["e%d" % lev])
            self._conv_bwd(a_, A[up], dz2[lev], D, G[up])
            Dc = D // 2
            self._ck(L.tbsg_up2_bwd_act(self._ptr(G[up]), self._ptr(A[ynext]), self._ptr(dz[lev + 1]), cn, self.B,
                                        Dc, Dc, Dc, SLOPE, st), "up_bwd_act")
        # bottleneck
        self._conv_bwd_act("e3c", A["e3b"], dz[3], s3, A["e3b"], dz2[3])
        self._conv_bwd_act("e3b", A["e3a"], dz2[3], s3, A["e3a"], dz[3])
        self._conv_bwd("e3a", A["p3"], dz[3], s3, G["p3"])
        self._ck(L.tbsg_pool2_bwd_act(self._ptr(G["p3"]), self._ptr(G["e2"]), self._ptr(A["e2"]), self._ptr(dz[2]), 64,
                                      self.B, s2, s2, s2, SLOPE, st), "pool_bwd_act")
        # encoder: level 2, 1, 0
        for lev, D, (b, a_), pin, cfine in ((2, s2, ("e2b", "e2a"), "p2", 32), (1, s1, ("e1b", "e1a"), "p1", 16),
                                            (0, s0, ("e0b", "e0a"), "x0", None)):
            self._conv_bwd_act(b, A[a_], dz[lev], D, A[a_], dz2[lev])
            self._conv_bwd(a_, A[pin], dz2[lev], D, G[pin] if cfine else None)
            if cfine:
                fine = "e%d" % (lev - 1)
                self._ck(L.tbsg_pool2_bwd_act(self._ptr(G[pin]), self._ptr(G[fine]), self._ptr(A[fine]),
                                              self._ptr(dz[lev - 1]), cfine, self.B, 2 * D, 2 * D, 2 * D, SLOPE, st),
                         "pool_bwd_act")
        return self.head_out[0:1]

    def adam_step(self, lr: float, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0, max_norm: float = 1.0):
        """One Adam step on the gradient of the last backward(), clipped to
        global norm `max_norm` on the device (no host round trip)."""
        self.step_t += 1
        self._ck(self.lib.tbsg_clip_scale(self._ptr(self.g), self.np, max_norm, self._ptr(self.clip_part),
                                          self._ptr(self.clip_out), self._st()), "clip")
        self._ck(self.lib.tbsg_adam(self._ptr(self.p), self._ptr(self.g), self._ptr(self.m), self._ptr(self.v),
                                    self.np, lr, beta1, beta2, eps, weight_decay, self.step_t,
                                    self._ptr(self.clip_out[1:2]), self._st()), "adam")
        self.prep()

    # -- weights on disk -----------------------------------------------------------------
    def save(self, path: str, meta: dict | None = None):
        np.savez_compressed(path, params=self.p.cpu().numpy(), S=self.S, meta=np.array(repr(meta or {})))

    def load(self, path: str):
        d = np.load(path)
        if d["params"].size != self.np:
            raise ValueError("parameter count mismatch")
        self.p.copy_(self.t.from_numpy(d["params"]))
        self.prep()


# ---- data: ground states from the batched solver -------------------------------------

def _tf_noise(b, i, ini, noise=True):
    b.init_state(i, "tf_noise", seed=ini["seed"], amp=ini["amp"], r_tf2=ini["r_tf2"],
                 noise_amp=ini["noise_amp"] if noise else 0.0)


def phase_spread(psi: np.ndarray, frac: float = 0.1) -> float:
    """Largest deviation (rad) of the phase of psi from its global phase over
    the cells where |psi| >= frac * max|psi|: about zero for a real state up
    to a global phase (the vortex-free ground state), of order pi where
    vortices wind the phase."""
    p = psi.astype(np.complex128)
    a = np.abs(p)
    m = a >= frac * a.max()
    g = np.sum(p[m] * a[m])
    g = g / abs(g) if abs(g) > 0 else 1.0
    return float(np.max(np.abs(np.angle(p[m] * np.conj(g)))))


def axial_winding(psi: np.ndarray, radius_frac: float = 0.2) -> int:
    """Phase winding number of psi around the trap axis (z through the grid
    centre) on a circle of radius radius_frac * nx cells in the middle z
    plane: the net number of vortex lines the circle encloses (0 for a
    vortex-free state), from bilinear samples of psi."""
    nx, ny, nz = psi.shape
    pl = psi[:, :, nz // 2].astype(np.complex128)
    cx, cy, r = (nx - 1) / 2.0, (ny - 1) / 2.0, radius_frac * nx
    t = np.linspace(0.0, 2 * np.pi, 8 * nx, endpoint=False)
    x, y = cx + r * np.cos(t), cy + r * np.sin(t)
    i0, j0 = np.floor(x).astype(int), np.floor(y).astype(int)
    fx, fy = x - i0, y - j0
    v = (pl[i0, j0] * (1 - fx) * (1 - fy) + pl[i0 + 1, j0] * fx * (1 - fy) + pl[i0, j0 + 1] * (1 - fx) * fy +
         pl[i0 + 1, j0 + 1] * fx * fy)
    d = np.angle(np.roll(v, -1) * np.conj(v))
    return int(round(float(np.sum(d)) / (2 * np.pi)))


def ground_states(draws, max_steps: int, tol: float, frac: float = 0.6, chunk: int = 32, omega_zero: bool = True):
    """Relax each draw from its Thomas-Fermi + noise guess with the batched
    RK3 solver at `frac` of its own stability limit (the fixed point does not
    depend on the step) and return the amplitudes |psi| (FP32) and stats.

    omega_zero: relax without the rotation term.  In these axisymmetric traps a
    real, current-free state has <Lz> = 0, so the vortex-free stationary state
    of the rotating frame -- the state an imaginary-time relaxation from the
    vortex-free guesses settles in before any vortex nucleates -- is the
    non-rotating ground state; relaxing at Omega = 0 gives that target without
    the symmetry-broken vortex states a long rotating relaxation can reach."""
    from .batch import BatchSolver
    amps, info = [], []
    for c0 in range(0, len(draws), chunk):
        part = draws[c0:c0 + chunk]
        ps = []
        for prob, _ in part:
            q = units.TrapProblem(n=prob.n, box=prob.box, omega=prob.omega, g=prob.g, mu=prob.mu,
                                  dt=stable_dtau(prob, frac), Omega=0.0 if omega_zero else prob.Omega,
                                  precision=prob.precision)
            ps.append(q.to_params())
        b = BatchSolver(ps)
        for i, (_, ini) in enumerate(part):
            _tf_noise(b, i, ini)
        out = b.solve(max_steps=max_steps, tol=tol, check_every=200)
        for i in range(len(part)):
            psi = b.get_psi(i)
            amps.append(np.abs(psi).astype(np.float32))
            st = b.status(i)
            info.append({"steps": out["steps"][i], "rel": st["rel"], "converged": st["converged"] > 0,
                         "phase_spread": phase_spread(psi)})
        b.close()
    return amps, info


def azimuthal_average(a: np.ndarray) -> np.ndarray:
    """The amplitude averaged over rotations about the trap axis (z through
    the grid centre), per z plane: means over rings of width one cell,
    linearly interpolated back to the cells by radius."""
    nx, ny, nz = a.shape
    x = np.arange(nx) - (nx - 1) / 2.0
    y = np.arange(ny) - (ny - 1) / 2.0
    r = np.sqrt(x[:, None] ** 2 + y[None, :] ** 2).ravel()
    b = np.floor(r).astype(np.int64)
    nb = b.max() + 1
    cnt = np.bincount(b, minlength=nb).astype(np.float64)
    rmean = np.bincount(b, weights=r, minlength=nb) / np.maximum(cnt, 1)
    flat = a.reshape(nx * ny, nz).astype(np.float64)
    out = np.empty_like(flat)
    for k in range(nz):
        m = np.bincount(b, weights=flat[:, k], minlength=nb) / np.maximum(cnt, 1)
        out[:, k] = np.interp(r, rmean, m)
    return out.reshape(a.shape).astype(a.dtype)


def training_target(amp: np.ndarray, vortex_dev: float = 0.1) -> tuple[np.ndarray, bool]:
    """A ground-state amplitude as a training target: states that deviate
    from their azimuthal average by more than `vortex_dev` somewhere carry
    vortices at symmetry-broken positions no amplitude predictor can learn,
    and are replaced by that average."""
    av = azimuthal_average(amp)
    if np.max(np.abs(amp - av)) > vortex_dev:
        return av, True
    return amp, False


# ---- training -----------------------------------------------------------------------------

def train(net: Surrogate, X, BASE, Y, epochs: int, lr: float = 5e-4, lr_min: float = 5e-6, seed: int = 0,
          warmup: int = 100, max_norm: float = 1.0, log=None) -> list[float]:
    """Adam over the resident dataset (X [N,S,S,S,16] BF16, BASE and Y
    [N,S,S,S] FP32, all on the device): linear warm-up over `warmup` steps,
    then a cosine decay to lr_min; gradients clipped to global norm max_norm."""
    t = net.t
    N = X.shape[0]
    rng = np.random.default_rng(seed)
    steps_per_epoch = max(1, N // net.B)
    total = epochs * steps_per_epoch
    hist = []
    k = 0
    for ep in range(epochs):
        order = rng.permutation(N)
        acc = t.zeros(1, dtype=t.float32, device=net.dev)
        for s in range(steps_per_epoch):
            idx = t.from_numpy(order[s * net.B:(s + 1) * net.B].copy()).to(net.dev)
            net.forward(X.index_select(0, idx), BASE.index_select(0, idx))
            acc += net.backward(Y.index_select(0, idx))
            if k < warmup:
                cur = lr * (k + 1) / warmup
            else:
                cur = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * (k - warmup) / max(1, total - warmup)))
            net.adam_step(cur, max_norm=max_norm)
            k += 1
        hist.append(float(acc.item()) / steps_per_epoch)
        if log:
            log(f"epoch {ep + 1}/{epochs} loss {hist[-1]:.3e}")
    return hist


def predict(net: Surrogate, feats: list[np.ndarray], bases: list[np.ndarray]) -> list[np.ndarray]:
    t = net.t
    out = []
    for i in range(0, len(feats), net.B):
        fb = feats[i:i + net.B]
        bb = bases[i:i + net.B]
        while len(fb) < net.B:   # pad the last batch
            fb = fb + [fb[-1]]
            bb = bb + [bb[-1]]
        x = t.from_numpy(np.stack(fb)).to(net.dev)
        base = t.from_numpy(np.stack(bb)).to(net.dev)
        amp = net.forward(x, base)
        res = amp.cpu().numpy()
        out.extend([np.maximum(res[j], 0.0) for j in range(min(net.B, len(feats) - i))])
    return out


def predict_problems(net: Surrogate, probs) -> tuple[list[np.ndarray], list[np.ndarray]]:
    """Predicted amplitudes (host, clipped at 0) and Thomas-Fermi bases (host)
    of the problems, with the input features built on the device."""
    t = net.t
    S = net.S
    x = t.empty((net.B, S, S, S, NFEAT), dtype=t.bfloat16, device=net.dev)
    base = t.empty((net.B, S, S, S), dtype=t.float32, device=net.dev)
    st = net._st()
    amps, bases = [], []
    for i in range(0, len(probs), net.B):
        pb = list(probs[i:i + net.B])
        while len(pb) < net.B:   # pad the last batch
            pb.append(pb[-1])
        for j, prob in enumerate(pb):
            features_device(net.lib, prob, x[j], base[j], st)
        amp = net.forward(x, base)
        res = amp.cpu().numpy()
        bh = base.cpu().numpy()
        k = min(net.B, len(probs) - i)
        amps.extend([np.maximum(res[j], 0.0) for j in range(k)])
        bases.extend([bh[j].copy() for j in range(k)])
    return amps, bases


# ---- the comparison: NN guess against the Thomas-Fermi guess ---------------------------------------

def _guesses(draws, amps, nn_noise: float):
    """Host copies of the two initial states per draw: the Thomas-Fermi guess
    with its seeded 1e-2 noise (the plain method) and the NN amplitude with
    the same seeded noise pattern scaled to `nn_noise`, given the TF guess's
    norm (the solver keeps the norm of its initial state)."""
    from .batch import BatchSolver
    b = BatchSolver([prob.to_params() for prob, _ in draws])
    tf, nn = [], []
    for i, (_, ini) in enumerate(draws):
        _tf_noise(b, i, ini)
        noisy = b.get_psi(i)
        _tf_noise(b, i, ini, noise=False)
        clean = b.get_psi(i)
        scale = nn_noise / ini["noise_amp"] if ini["noise_amp"] > 0 else 0.0
        guess = amps[i] + (noisy - clean) * scale
        n_tf = np.sum(np.abs(noisy.astype(np.complex128)) ** 2)
        n_nn = np.sum(np.abs(guess.astype(np.complex128)) ** 2)
        tf.append(noisy)
        nn.append((guess * math.sqrt(n_tf / n_nn)).astype(noisy.dtype))
    b.close()
    return tf, nn


def _relax(params, states, tol, max_steps, check_every, energy_only=False, escale=None, keep_finals=True):
    """Batched RK3_RENORM relaxation of `states`; with `escale` (one per state)
    the stop test is |dE| / N * escale < tol (trapbec_batch_set_imag_stop
    ABS_PER_NORM), else |dE|/|E| <= tol."""
    from .batch import BatchSolver
    b = BatchSolver(params)
    for i, s in enumerate(states):
        b.set_psi(i, s)
    if escale is not None and not energy_only:
        b.set_imag_stop(abi.STOP_ABS_PER_NORM, escale)
    t0 = time.perf_counter()
    out = b.solve(max_steps=1 if energy_only else max_steps, tol=0.0 if energy_only else tol,
                  check_every=check_every)
    wall = time.perf_counter() - t0
    st = b.stats()
    res = {"steps": out["steps"], "energy": out["energy"],
           "converged": [b.status(i)["converged"] > 0 for i in range(len(states))],
           "solve_ms_device": st["solve_ms"], "wall_s": wall}
    finals = None if energy_only or not keep_finals else [b.get_psi(i) for i in range(len(states))]
    b.close()
    return res, finals


def compare(net: Surrogate, draws, tol: float = 1e-10, max_steps: int = 60000, check_every: int = 200,
            nn_noise: float = 1e-2, nn_omega_max: float = 0.5, stop: str = "rel", subset_rerun: bool = False) -> dict:
    """Relax the held-out draws twice at the workload's step (dtau = 0.002):
    from the Thomas-Fermi + 1e-2 noise guess (the plain method) and with the
    surrogate.  The surrogate's initial state is its amplitude plus the same
    seeded noise pattern at `nn_noise`, unless the Thomas-Fermi guess has the
    lower energy at the same norm (or the prediction is unreasonable), in
    which case the Thomas-Fermi guess is the fallback.  Above Omega/omega_perp
    = `nn_omega_max` the Thomas-Fermi guess is always kept: there the
    relaxation is bistable -- from the Thomas-Fermi guess it can nucleate
    vortices and end in a vortex state 10-20% lower in energy, from the
    surrogate's guess (close to the vortex-free stationary state) it stops
    there -- so the two guesses would not lead to the same state.  Reports steps and
    device time to the energy-change tolerance -- relative, |dE|/|E| <= tol
    (stop="rel"), or on the energy per particle in trap units, |d(E/N)| < tol
    (stop="per_particle") -- the final energies and the L2 distance of the
    final states (global phase aligned), and the phase winding of each final
    state around the trap axis (nonzero where the relaxation ended with
    vortices).  With `subset_rerun`, the draws whose plain relaxation reaches
    the tolerance are relaxed again in both arms as batches of their own, so
    that the batch wall-time ratio of that set is not set by the draws that
    never converge (which keep the Thomas-Fermi guess and run max_steps in
    both arms)."""
    t = net.t
    escale = [prob.mu_to_trap(1.0) for prob, _ in draws] if stop == "per_particle" else None
    params = [prob.to_params() for prob, _ in draws]
    probs = [prob for prob, _ in draws]
    predict_problems(net, probs[:net.B])   # warm-up
    ev0, ev1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
    t.cuda.synchronize()
    ev0.record()
    amps, bases = predict_problems(net, probs)   # features on the device, amplitudes back on the host
    ev1.record()
    t.cuda.synchronize()
    infer_ms = ev0.elapsed_time(ev1)
    unreasonable = []
    for i, (a_, base_) in enumerate(zip(amps, bases)):
        rms = float(np.sqrt(np.mean((a_ - base_) ** 2)))
        bad = not np.all(np.isfinite(a_)) or rms > 0.25 or a_.max() > 1.5
        unreasonable.append(bad)
        if bad:
            amps[i] = base_
    tf_states, nn_states = _guesses(draws, amps, nn_noise)
    # the selector: the guess with the lower energy at the same norm
    e_tf, _ = _relax(params, tf_states, tol, max_steps, check_every, energy_only=True)
    e_nn, _ = _relax(params, nn_states, tol, max_steps, check_every, energy_only=True)
    slow_rot = [prob.Omega <= nn_omega_max * prob.omega[0] for prob, _ in draws]
    use_nn = [(not bad) and ok and en < et
              for bad, ok, en, et in zip(unreasonable, slow_rot, e_nn["energy"], e_tf["energy"])]
    sel_ms = e_tf["solve_ms_device"] + e_nn["solve_ms_device"]   # the selector's energy evaluations
    chosen = [n if u else f for n, f, u in zip(nn_states, tf_states, use_nn)]
    res, finals = {}, {}
    res["tf"], finals["tf"] = _relax(params, tf_states, tol, max_steps, check_every, escale=escale)
    res["nn"], finals["nn"] = _relax(params, chosen, tol, max_steps, check_every, escale=escale)
    l2 = []
    for a, c in zip(finals["tf"], finals["nn"]):
        a = a.astype(np.complex128).ravel()
        c = c.astype(np.complex128).ravel()
        ph = np.vdot(c, a)
        ph = ph / abs(ph) if abs(ph) > 0 else 1.0
        l2.append(float(np.linalg.norm(a - c * ph) / np.linalg.norm(a)))
    wind_tf = [axial_winding(f) for f in finals["tf"]]
    wind_nn = [axial_winding(f) for f in finals["nn"]]
    subset = None
    sub = [i for i, c in enumerate(res["tf"]["converged"]) if c]
    if subset_rerun and sub and len(sub) < len(draws):
        pick = lambda v: [v[i] for i in sub] if v is not None else None
        r_tf, _ = _relax(pick(params), pick(tf_states), tol, max_steps, check_every, escale=pick(escale),
                         keep_finals=False)
        r_nn, _ = _relax(pick(params), pick(chosen), tol, max_steps, check_every, escale=pick(escale),
                         keep_finals=False)
        share = len(sub) / len(draws)   # this set's share of the inference and the selector
        subset = {"instances": len(sub), "nn_used": int(sum(use_nn[i] for i in sub)),
                  "converged_tf": int(sum(r_tf["converged"])), "converged_nn": int(sum(r_nn["converged"])),
                  "device_ms_tf": r_tf["solve_ms_device"], "device_ms_nn": r_nn["solve_ms_device"],
                  "steps_tf": r_tf["steps"], "steps_nn": r_nn["steps"],
                  "wall_ratio_device": r_tf["solve_ms_device"] /
                                       (r_nn["solve_ms_device"] + share * (infer_ms + sel_ms))}
    de = [abs(x - y) / abs(x) for x, y in zip(res["tf"]["energy"], res["nn"]["energy"])]
    rms = lambda a, b: float(np.sqrt(np.mean((a - b) ** 2)))
    s_tf, s_nn = np.array(res["tf"]["steps"], float), np.array(res["nn"]["steps"], float)
    both = np.array([a and b for a, b in zip(res["tf"]["converged"], res["nn"]["converged"])])
    ratio = s_tf / np.maximum(s_nn, 1)
    return {
        "instances": len(draws), "tol": tol, "stop": stop, "dtau_trap_units": draws[0][0].dt, "nn_noise": nn_noise,
        "nn_used": int(sum(use_nn)), "nn_unreasonable": int(sum(unreasonable)),
        "nn_omega_max": nn_omega_max, "tf_kept_fast_rotation": int(len(draws) - sum(slow_rot)),
        "guess_energy_tf": e_tf["energy"], "guess_energy_nn": e_nn["energy"],
        "tf": res["tf"], "nn": res["nn"], "nn_inference_ms": infer_ms,
        "steps_ratio_per_instance": ratio.tolist(),
        "steps_ratio_median": float(np.median(ratio)),
        "steps_ratio_median_nn_used": float(np.median(ratio[np.array(use_nn)])) if any(use_nn) else None,
        "steps_ratio_total": float(s_tf.sum() / max(s_nn.sum(), 1)),
        "steps_ratio_total_both_converged": float(s_tf[both].sum() / max(s_nn[both].sum(), 1)) if both.any() else None,
        "selection_ms_device": sel_ms,
        "wall_ratio_device": res["tf"]["solve_ms_device"] / (res["nn"]["solve_ms_device"] + infer_ms + sel_ms),
        "final_energy_rel_diff_max": float(max(de)), "final_l2_rel": l2,
        "same_end_state": int(sum(x <= 1e-4 for x in de)),   # |dE|/|E| <= 1e-4 between the two final states
        "guess_rmse_tf": [rms(np.abs(f), b_) for f, b_ in zip(finals["tf"], bases)],
        "guess_rmse_nn": [rms(np.abs(f), a_) for f, a_ in zip(finals["tf"], amps)],
        "winding_tf": wind_tf, "winding_nn": wind_nn,
        "omega_over_omega_perp": [prob.Omega / prob.omega[0] for prob, _ in draws],
        "subset_tf_converged": subset,
    }


def holdout_error(net: Surrogate, probs, targets) -> dict:
    """Error of the network's amplitude (and of the Thomas-Fermi amplitude)
    against held-out ground-state amplitudes: RMS over the grid per draw."""
    amps, bases = predict_problems(net, probs)
    rms = lambda x, y: float(np.sqrt(np.mean((x.astype(np.float64) - y) ** 2)))
    e_nn = np.array([rms(x, t) for x, t in zip(amps, targets)])
    e_tf = np.array([rms(b, t) for b, t in zip(bases, targets)])
    return {"holdout": len(targets), "holdout_rmse_nn_median": float(np.median(e_nn)),
            "holdout_rmse_nn_mean": float(np.mean(e_nn)), "holdout_rmse_tf_median": float(np.median(e_tf)),
            "holdout_rmse_ratio_tf_over_nn_median": float(np.median(e_tf / np.maximum(e_nn, 1e-30)))}


# ---- command line: generate, train, compare ----------------------------------------------------

def conv_flops(S: int, batch: int) -> tuple[float, float]:
    """FLOPs of the convolutions of one forward pass and of one backward pass
    (input gradients for every layer but the first, weight gradients for all)."""
    lev = [0, 0, 1, 1, 2, 2, 3, 3, 3, 2, 2, 1, 1, 0, 0]
    fwd = sum(2.0 * 27 * ci * co * batch * (S >> l) ** 3 for (_, ci, co), l in zip(LAYERS, lev))
    first = 2.0 * 27 * 16 * 16 * batch * S ** 3
    return fwd, 2 * fwd - first


def time_passes(S: int, batch: int, reps: int) -> dict:
    """Device time of forward and forward+backward+Adam passes (random weights
    and inputs) and the tensor-core rate of the convolutions."""
    torch = _torch()
    net = Surrogate(S, batch, seed=1)
    net.p[-(NFEAT + 1):].copy_(torch.linspace(-0.5, 0.5, NFEAT + 1))
    net.prep()
    g = torch.Generator(device="cpu").manual_seed(0)
    x = torch.randn((batch, S, S, S, NFEAT), generator=g).to(net.dev).to(torch.bfloat16)
    base = torch.rand((batch, S, S, S), generator=g).to(net.dev)
    tgt = base + 0.05
    for _ in range(2):
        net.forward(x, base)
        net.backward(tgt)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    e[0].record()
    for _ in range(reps):
        net.forward(x, base)
    e[1].record()
    for _ in range(reps):
        net.forward(x, base)
        net.backward(tgt)
        net.adam_step(1e-6)
    e[2].record()
    torch.cuda.synchronize()
    f_ms = e[0].elapsed_time(e[1]) / reps
    t_ms = e[1].elapsed_time(e[2]) / reps
    ff, fb = conv_flops(S, batch)
    return {"S": S, "batch": batch, "forward_ms": f_ms, "train_step_ms": t_ms,
            "conv_tflops_forward": ff / (f_ms * 1e-3) / 1e12,
            "conv_tflops_train_step": (ff + fb) / (t_ms * 1e-3) / 1e12,
            "conv_gflop_forward": ff / 1e9, "conv_gflop_backward": fb / 1e9}


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="train the warm-start surrogate on solver ground states and compare "
                                             "imaginary-time relaxation from its guess against the TF guess")
    ap.add_argument("--S", type=int, default=128, help="grid (S^3)")
    ap.add_argument("--n-train", type=int, default=192)
    ap.add_argument("--n-test", type=int, default=16)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--gen-steps", type=int, default=8000, help="relaxation steps per training ground state")
    ap.add_argument("--gen-frac", type=float, default=0.85, help="fraction of the RK3 stability limit for data")
    ap.add_argument("--target-omega", choices=["zero", "draw"], default="zero",
                    help="training ground states relaxed without rotation (the vortex-free stationary state) "
                         "or at each draw's Omega")
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--batch", type=int, default=2)
    ap.add_argument("--lr", type=float, default=5e-4)
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--max-steps", type=int, default=60000)
    ap.add_argument("--nn-noise", type=float, nargs="+", default=[1e-2],
                    help="noise level(s) of the NN guess (the TF guess keeps 1e-2)")
    ap.add_argument("--weights", default=None, help="load weights instead of training")
    ap.add_argument("--symmetrize", type=int, default=0,
                    help="train vortex states on their azimuthal average (1) or as they are (0)")
    ap.add_argument("--out", default=None, help="save the trained weights (.npz)")
    ap.add_argument("--json", default=None)
    ap.add_argument("--time", type=int, default=0, metavar="REPS",
                    help="only time forward and training passes (random weights) and exit")
    ap.add_argument("--curve", type=int, nargs="*", default=[],
                    help="also train fresh networks on the first K training draws for the same number of optimizer "
                         "steps and report their held-out error (a learning curve)")
    ap.add_argument("--holdout-gs", type=int, default=0,
                    help="relax this many held-out draws to their ground states and report the guess error on them")
    ap.add_argument("--stop", choices=["rel", "per_particle"], default="per_particle",
                    help="stop test of the comparison: |dE|/|E| <= tol or |d(E/N)| < tol in trap units")
    ap.add_argument("--no-compare", action="store_true", help="skip the relaxation comparison")
    ap.add_argument("--subset-rerun", action="store_true",
                    help="also relax the draws whose TF relaxation converges as batches of their own")
    a = ap.parse_args(argv)
    if a.time:
        r = time_passes(a.S, a.batch, a.time)
        print(json.dumps(r), flush=True)
        if a.json:
            with open(a.json, "w") as f:
                json.dump(r, f, indent=1)
        return r
    torch = _torch()
    log = lambda m: print(m, flush=True)
    draws = units.ground_state_draws(a.n_train + a.n_test, a.seed, grids=(a.S,), precision=abi.FP32)
    train_d, test_d = draws[:a.n_train], draws[a.n_train:]
    net = Surrogate(a.S, a.batch, seed=a.seed)
    rep = {"S": a.S, "n_params": net.np, "n_train": a.n_train, "n_test": a.n_test, "seed": a.seed}
    if a.weights:
        net.load(a.weights)
        rep["weights"] = a.weights
    else:
        t0 = time.perf_counter()
        amps, info = ground_states(train_d, max_steps=a.gen_steps, tol=1e-12, frac=a.gen_frac,
                                   omega_zero=a.target_omega == "zero")
        rep["target_omega"] = a.target_omega
        rep["gen_s"] = time.perf_counter() - t0
        rep["gen_rel_dE_median"] = float(np.median([i["rel"] for i in info]))
        ps = [i["phase_spread"] for i in info]
        rep["gen_phase_spread_rad"] = {"median": float(np.median(ps)), "max": float(np.max(ps)),
                                       "note": "largest phase deviation from the global phase where "
                                               "|psi| >= 0.1 max|psi|, per training ground state"}
        log(f"generated {len(amps)} ground states in {rep['gen_s']:.1f} s, median rel dE {rep['gen_rel_dE_median']:.2e}, "
            f"phase spread median {rep['gen_phase_spread_rad']['median']:.1e} max {rep['gen_phase_spread_rad']['max']:.1e}")
        hold = None
        if a.holdout_gs and test_d:
            hd = test_d[:a.holdout_gs]
            hamps, hinfo = ground_states(hd, max_steps=a.gen_steps, tol=1e-12, frac=a.gen_frac,
                                         omega_zero=a.target_omega == "zero")
            hold = ([p for p, _ in hd], hamps)
            rep["holdout_gs"] = {"instances": len(hd),
                                 "phase_spread_rad_max": float(np.max([i["phase_spread"] for i in hinfo]))}
        X = torch.empty((a.n_train, a.S, a.S, a.S, NFEAT), dtype=torch.bfloat16, device=net.dev)
        BASE = torch.empty((a.n_train, a.S, a.S, a.S), dtype=torch.float32, device=net.dev)
        Y = torch.empty_like(BASE)
        n_vortex = 0
        for i, (prob, _) in enumerate(train_d):
            features_device(net.lib, prob, X[i], BASE[i])
            tgt, vort = training_target(amps[i]) if a.symmetrize else (amps[i], False)
            n_vortex += vort
            Y[i].copy_(torch.from_numpy(tgt))
        rep["targets_symmetrized"] = n_vortex
        rep["tf_guess_rmse"] = float(torch.sqrt(((BASE - Y) ** 2).mean()).item())
        total_steps = a.epochs * max(1, a.n_train // a.batch)
        curve = []
        for k in sorted(set(x for x in a.curve if 0 < x < a.n_train)):
            nk = Surrogate(a.S, a.batch, seed=a.seed)
            ek = max(1, round(total_steps / max(1, k // a.batch)))
            t0 = time.perf_counter()
            hk = train(nk, X[:k], BASE[:k], Y[:k], epochs=ek, lr=a.lr, lr_min=a.lr * 1e-2, seed=a.seed)
            torch.cuda.synchronize()
            ent = {"n_train": k, "epochs": ek, "steps": nk.step_t, "train_s": time.perf_counter() - t0,
                   "loss_last": hk[-1]}
            if hold:
                ent.update(holdout_error(nk, *hold))
            curve.append(ent)
            log(json.dumps(ent))
            del nk
        t0 = time.perf_counter()
        hist = train(net, X, BASE, Y, epochs=a.epochs, lr=a.lr, lr_min=a.lr * 1e-2, seed=a.seed, log=log)
        rep["loss_history"] = hist
        torch.cuda.synchronize()
        rep["train_s"] = time.perf_counter() - t0
        rep["train_steps"] = net.step_t
        rep["loss_first"], rep["loss_last"] = hist[0], hist[-1]
        rep["train_rmse"] = math.sqrt(hist[-1])
        del X, BASE, Y
        ent = {"n_train": a.n_train, "epochs": a.epochs, "steps": net.step_t, "train_s": rep["train_s"],
               "loss_last": hist[-1]}
        if hold:
            ent.update(holdout_error(net, *hold))
        curve.append(ent)
        log(json.dumps(ent))
        rep["learning_curve"] = curve
        if a.out:
            net.save(a.out, {"S": a.S, "n_train": a.n_train, "seed": a.seed, "epochs": a.epochs})
    # held-out accuracy of the guess itself, then the relaxation comparison
    rep["compare"] = []
    for nz in (a.nn_noise if test_d and not a.no_compare else []):
        cmp_ = compare(net, test_d, tol=a.tol, max_steps=a.max_steps, nn_noise=nz, stop=a.stop,
                       subset_rerun=a.subset_rerun)
        rep["compare"].append(cmp_)
        log(json.dumps({k: cmp_[k] for k in ("nn_noise", "nn_used", "steps_ratio_median", "steps_ratio_median_nn_used",
                                              "steps_ratio_total", "steps_ratio_total_both_converged",
                                              "wall_ratio_device", "final_energy_rel_diff_max", "same_end_state",
                                              "tf_kept_fast_rotation")}))
        if cmp_["subset_tf_converged"]:
            log(json.dumps({"subset_tf_converged": {k: v for k, v in cmp_["subset_tf_converged"].items()
                                                    if not k.startswith("steps")}}))
    if a.json:
        with open(a.json, "w") as f:
            json.dump(rep, f, indent=1)
    return rep


if __name__ == "__main__":
    main()
