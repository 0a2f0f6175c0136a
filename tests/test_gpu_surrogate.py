"""The warm-start surrogate's kernels against the CPU oracle (float64
PyTorch on the CPU, fed the same BF16-rounded operands).

Tolerances: FP32-output convolutions and weight gradients accumulate exact
BF16 products in FP32 -> 1e-5 relative to the largest value; BF16 outputs
-> one BF16 rounding (2^-8 relative).

The whole network is checked twice.  (1) Layer by layer, from the GPU's own
stored activations and upstream gradients: every weight, bias and activation
gradient, skip sum, pooling and upsampling gradient is recomputed in float64
and must match to 1e-5 (the BF16 rounding of each dz is reproduced exactly).
(2) End to end against the float64 oracle: forward activations drift by a
few 1e-3 with depth (BF16 rounding flips compound), and where that drift
changes the sign of a pre-activation the leaky ReLU's derivative jumps from
1 to 0.05, so gradients agree only to about 5%; the bounds are loss 1e-3 and
1.5e-1 per layer."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import nn_oracle
from trapbec_gb300 import abi
from trapbec_gb300.surrogate import LAYERS, NFEAT, Surrogate, n_params, train

pytestmark = pytest.mark.gpu

PAIRS = [(16, 16), (16, 32), (32, 16), (32, 32), (32, 64), (64, 32), (64, 64), (64, 128), (128, 64), (128, 128)]


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _bf(a, dev="cuda"):
    return torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).to(dev)


@pytest.fixture(params=[0, 1], ids=["tcgen05", "mma_sync"])
def conv_path(request):
    """Kernel family of tbsg_conv3_fwd: 0 = tcgen05 for 16/32 -> 16/32
    channels (mma.sync for the rest), 1 = mma.sync everywhere."""
    lib = abi.load()
    assert lib.tbsg_set_conv_path(request.param) == 0
    yield request.param
    assert lib.tbsg_set_conv_path(0) == 0
    flag = C.c_int(-1)
    assert lib.tbsg_tc_status(C.byref(flag)) == 0 and flag.value == 0


@pytest.mark.parametrize("cin,cout", PAIRS)
def test_conv3_forward_and_gradients(cin, cout, conv_path):
    lib = abi.load()
    rng = np.random.default_rng(cin * 1000 + cout)
    B, D, H, W = 2, 3, 10, 12          # partial bricks in every direction
    xb = _bf(rng.normal(size=(B, D, H, W, cin)))
    wb = _bf(rng.normal(size=(27, cout, cin)) / np.sqrt(27 * cin))
    dzb = _bf(rng.normal(size=(B, D, H, W, cout)))
    x64, w64, dz64 = (t.double().cpu() for t in (xb, wb, dzb))
    bias = torch.tensor(rng.normal(size=cout), dtype=torch.float32, device="cuda")
    skip = _bf(rng.normal(size=(B, D, H, W, cout)))
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # FP32 output
    yf = torch.empty((B, D, H, W, cout), dtype=torch.float32, device="cuda")
    assert lib.tbsg_conv3_fwd(_p(xb), cin, _p(wb), None, None, None, _p(yf), 0, cout, B, D, H, W, 0, 0.0, st) == 0
    ref = nn_oracle.conv3(x64, w64)
    assert (yf.double().cpu() - ref).abs().max() <= 1e-5 * ref.abs().max()
    # accumulate mode adds
    assert lib.tbsg_conv3_fwd(_p(xb), cin, _p(wb), None, None, None, _p(yf), 1, cout, B, D, H, W, 0, 0.0, st) == 0
    assert (yf.double().cpu() - 2 * ref).abs().max() <= 2e-5 * ref.abs().max()
    # BF16 output with bias, skip and the leaky ReLU
    y = torch.empty((B, D, H, W, cout), dtype=torch.bfloat16, device="cuda")
    assert lib.tbsg_conv3_fwd(_p(xb), cin, _p(wb), _p(bias), _p(skip), _p(y), None, 0, cout, B, D, H, W, 1, 0.05,
                              st) == 0
    ref2 = nn_oracle.act(ref + bias.double().cpu() + skip.double().cpu())
    assert (y.double().cpu() - ref2).abs().max() <= 2 ** -7 * ref2.abs().max()
    # input gradient: the forward pass of the flipped, transposed kernel
    w32 = wb.float()
    wk = torch.empty_like(wb)
    wt = torch.empty_like(wb)
    assert lib.tbsg_weight_prep(_p(w32), _p(wk), _p(wt), cin, cout, st) == 0
    assert torch.equal(wk, wb)
    gx = torch.empty((B, D, H, W, cin), dtype=torch.float32, device="cuda")
    assert lib.tbsg_conv3_fwd(_p(dzb), cout, _p(wt), None, None, None, _p(gx), 0, cin, B, D, H, W, 0, 0.0, st) == 0
    xr = x64.clone().requires_grad_(True)
    wr = w64.clone().requires_grad_(True)
    out = nn_oracle.conv3(xr, wr, torch.zeros(cout, dtype=torch.float64, requires_grad=True))
    (out * dz64).sum().backward()
    assert (gx.double().cpu() - xr.grad).abs().max() <= 1e-5 * xr.grad.abs().max()
    # the input gradient fused with the activation derivative below: bit for bit the two-step result
    yin = _bf(rng.normal(size=(B, D, H, W, cin)))
    dz_ref = torch.empty((B, D, H, W, cin), dtype=torch.bfloat16, device="cuda")
    sk_ref = torch.tensor(rng.normal(size=(B, D, H, W, cin)), dtype=torch.float32, device="cuda")
    sk = sk_ref.clone()
    assert lib.tbsg_act_bwd(_p(gx), _p(yin), _p(dz_ref), _p(sk_ref), gx.numel(), 0.05, st) == 0
    dz_in = torch.empty_like(dz_ref)
    assert lib.tbsg_conv3_dgrad_act(_p(dzb), cout, _p(wt), _p(yin), _p(dz_in), _p(sk), cin, B, D, H, W, 0.05, st) == 0
    assert torch.equal(dz_in.view(torch.int16), dz_ref.view(torch.int16))
    assert torch.equal(sk, sk_ref)
    # weight and bias gradients
    dw = torch.empty((27, cout, cin), dtype=torch.float32, device="cuda")
    db = torch.empty(cout, dtype=torch.float32, device="cuda")
    sb = lib.tbsg_conv3_wgrad_scratch_bytes(cin, cout, B, D, H, W)
    scr = torch.empty(sb // 4 + 1, dtype=torch.float32, device="cuda")
    assert lib.tbsg_conv3_wgrad(_p(xb), cin, _p(dzb), cout, B, D, H, W, _p(dw), _p(db), _p(scr), sb, st) == 0
    assert (dw.double().cpu() - wr.grad).abs().max() <= 1e-5 * wr.grad.abs().max()
    assert (db.double().cpu() - dz64.sum(dim=(0, 1, 2, 3))).abs().max() <= 1e-5 * dz64.abs().sum(dim=(0, 1, 2, 3)).max()
    # deterministic
    dw2 = torch.empty_like(dw)
    assert lib.tbsg_conv3_wgrad(_p(xb), cin, _p(dzb), cout, B, D, H, W, _p(dw2), None, _p(scr), sb, st) == 0
    assert torch.equal(dw, dw2)


@pytest.mark.parametrize("cin,cout", [(32, 64), (64, 32), (64, 64), (64, 128), (128, 64), (128, 128)])
def test_streamed_weight_kernel_two_brick_units(cin, cout):
    """The 64/128-channel tensor-core kernel on a grid with enough bricks for
    units of two bricks sharing each weight slice (partial bricks in h and w,
    a pair whose second brick lies outside the grid): forward against the
    oracle, and the fused input-gradient epilogue bit for bit against the
    two-step result."""
    lib = abi.load()
    assert lib.tbsg_set_conv_path(0) == 0
    rng = np.random.default_rng(cin + 7 * cout)
    B, D, H, W = 2, 20, 20, 20      # 160 two-brick units (>= the SM count)
    xb = _bf(rng.normal(size=(B, D, H, W, cin)))
    wb = _bf(rng.normal(size=(27, cout, cin)) / np.sqrt(27 * cin))
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    yf = torch.empty((B, D, H, W, cout), dtype=torch.float32, device="cuda")
    assert lib.tbsg_conv3_fwd(_p(xb), cin, _p(wb), None, None, None, _p(yf), 0, cout, B, D, H, W, 0, 0.0, st) == 0
    ref = nn_oracle.conv3(xb.double().cpu(), wb.double().cpu())
    assert (yf.double().cpu() - ref).abs().max() <= 1e-5 * ref.abs().max()
    yact = _bf(rng.normal(size=(B, D, H, W, cout)))
    dz_ref = torch.empty((B, D, H, W, cout), dtype=torch.bfloat16, device="cuda")
    assert lib.tbsg_act_bwd(_p(yf), _p(yact), _p(dz_ref), None, yf.numel(), 0.05, st) == 0
    dz = torch.empty_like(dz_ref)
    assert lib.tbsg_conv3_dgrad_act(_p(xb), cin, _p(wb), _p(yact), _p(dz), None, cout, B, D, H, W, 0.05, st) == 0
    assert torch.equal(dz.view(torch.int16), dz_ref.view(torch.int16))
    flag = C.c_int(-1)
    assert lib.tbsg_tc_status(C.byref(flag)) == 0 and flag.value == 0


def test_unsupported_pair_is_an_error():
    lib = abi.load()
    x = torch.zeros(16 * 8, dtype=torch.bfloat16, device="cuda")
    assert lib.tbsg_conv3_fwd(_p(x), 16, _p(x), None, None, _p(x), None, 0, 48, 1, 2, 2, 2, 0, 0.0, None) == 2


def test_pool_up_act_head_adam():
    lib = abi.load()
    rng = np.random.default_rng(5)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    B, D, c = 2, 6, 32
    x = _bf(rng.normal(size=(B, D, D, D, c)))
    y = torch.empty((B, D // 2, D // 2, D // 2, c), dtype=torch.bfloat16, device="cuda")
    assert lib.tbsg_pool2_fwd(_p(x), _p(y), c, B, D, D, D, st) == 0
    ref = nn_oracle.pool2(x.double().cpu())
    assert (y.double().cpu() - ref).abs().max() <= 2 ** -8 * ref.abs().max()
    u = torch.empty_like(x)
    assert lib.tbsg_up2_fwd(_p(y), _p(u), c, B, D // 2, D // 2, D // 2, st) == 0
    assert torch.equal(u, nn_oracle.up2(y.cpu()).cuda())
    g = torch.tensor(rng.normal(size=(B, D, D, D, c)), dtype=torch.float32, device="cuda")
    gc = torch.empty((B, D // 2, D // 2, D // 2, c), dtype=torch.float32, device="cuda")
    assert lib.tbsg_up2_bwd(_p(g), _p(gc), c, B, D // 2, D // 2, D // 2, st) == 0
    want = g.double().cpu().reshape(B, D // 2, 2, D // 2, 2, D // 2, 2, c).sum(dim=(2, 4, 6))
    assert (gc.double().cpu() - want).abs().max() <= 1e-5 * want.abs().max()
    acc = torch.ones_like(g)
    assert lib.tbsg_pool2_bwd(_p(gc), _p(acc), c, B, D, D, D, st) == 0
    want = 1.0 + nn_oracle.up2(gc.double().cpu()) / 8
    assert (acc.double().cpu() - want).abs().max() <= 1e-6 * want.abs().max()
    # activation gradient with the skip accumulation
    yb = _bf(rng.normal(size=1000))
    dy = torch.tensor(rng.normal(size=1000), dtype=torch.float32, device="cuda")
    dz = torch.empty(1000, dtype=torch.bfloat16, device="cuda")
    sk = torch.ones(1000, dtype=torch.float32, device="cuda")
    assert lib.tbsg_act_bwd(_p(dy), _p(yb), _p(dz), _p(sk), 1000, 0.05, st) == 0
    wantg = dy.double().cpu() * torch.where(yb.double().cpu() > 0, 1.0, 0.05)
    assert (dz.double().cpu() - wantg).abs().max() <= 2 ** -8 * wantg.abs().max()
    assert (sk.double().cpu() - 1 - wantg).abs().max() <= 1e-6 * wantg.abs().max()
    # head and loss
    n = 5000
    feat = _bf(rng.normal(size=(n, NFEAT)))
    wh = torch.tensor(rng.normal(size=NFEAT), dtype=torch.float32, device="cuda")
    bh = torch.tensor([0.3], dtype=torch.float32, device="cuda")
    base = torch.tensor(rng.uniform(size=n), dtype=torch.float32, device="cuda")
    tgt = torch.tensor(rng.uniform(size=n), dtype=torch.float32, device="cuda")
    dfeat = torch.empty((n, NFEAT), dtype=torch.float32, device="cuda")
    part = torch.empty(lib.tbsg_head_partials(n, NFEAT), dtype=torch.float32, device="cuda")
    out = torch.empty(NFEAT + 2, dtype=torch.float32, device="cuda")
    assert lib.tbsg_head_loss(_p(feat), NFEAT, _p(wh), _p(bh), _p(base), _p(tgt), n, _p(dfeat), _p(part), _p(out),
                              st) == 0
    f64 = feat.double().cpu()
    whr = wh.double().cpu().requires_grad_(True)
    bhr = bh.double().cpu().requires_grad_(True)
    fr = f64.clone().requires_grad_(True)
    loss = ((base.double().cpu() + fr @ whr + bhr - tgt.double().cpu()) ** 2).mean()
    loss.backward()
    o = out.double().cpu()
    assert abs(o[0] - loss.item()) <= 1e-5 * loss.item()
    assert (o[1:NFEAT + 1] - whr.grad).abs().max() <= 1e-5 * whr.grad.abs().max()
    assert abs(o[NFEAT + 1] - bhr.grad[0]) <= 1e-5 * abs(bhr.grad[0]) + 1e-7
    assert (dfeat.double().cpu() - fr.grad).abs().max() <= 1e-5 * fr.grad.abs().max()
    # the activation-gradient fusions: bit for bit the gradient kernel followed by act_bwd
    dzf = torch.empty((n, NFEAT), dtype=torch.bfloat16, device="cuda")
    dzr = torch.empty_like(dzf)
    out2 = torch.empty_like(out)
    assert lib.tbsg_act_bwd(_p(dfeat), _p(feat), _p(dzr), None, dfeat.numel(), 0.05, st) == 0
    assert lib.tbsg_head_loss_act(_p(feat), _p(wh), _p(bh), _p(base), _p(tgt), n, _p(dzf), 0.05, _p(part),
                                  _p(out2), st) == 0
    assert torch.equal(dzf.view(torch.int16), dzr.view(torch.int16)) and torch.equal(out2, out)
    yf_ = _bf(rng.normal(size=(B, D, D, D, c)))
    gfine = torch.tensor(rng.normal(size=(B, D, D, D, c)), dtype=torch.float32, device="cuda")
    acc = gfine.clone()
    assert lib.tbsg_pool2_bwd(_p(gc), _p(acc), c, B, D, D, D, st) == 0
    dzr = torch.empty((B, D, D, D, c), dtype=torch.bfloat16, device="cuda")
    assert lib.tbsg_act_bwd(_p(acc), _p(yf_), _p(dzr), None, acc.numel(), 0.05, st) == 0
    dzp = torch.empty_like(dzr)
    assert lib.tbsg_pool2_bwd_act(_p(gc), _p(gfine), _p(yf_), _p(dzp), c, B, D, D, D, 0.05, st) == 0
    assert torch.equal(dzp.view(torch.int16), dzr.view(torch.int16))
    yc_ = _bf(rng.normal(size=(B, D // 2, D // 2, D // 2, c)))
    gcs = torch.empty((B, D // 2, D // 2, D // 2, c), dtype=torch.float32, device="cuda")
    assert lib.tbsg_up2_bwd(_p(g), _p(gcs), c, B, D // 2, D // 2, D // 2, st) == 0
    dzr = torch.empty((B, D // 2, D // 2, D // 2, c), dtype=torch.bfloat16, device="cuda")
    assert lib.tbsg_act_bwd(_p(gcs), _p(yc_), _p(dzr), None, gcs.numel(), 0.05, st) == 0
    dzu = torch.empty_like(dzr)
    assert lib.tbsg_up2_bwd_act(_p(g), _p(yc_), _p(dzu), c, B, D // 2, D // 2, D // 2, 0.05, st) == 0
    assert torch.equal(dzu.view(torch.int16), dzr.view(torch.int16))
    # Adam
    p0 = torch.tensor(rng.normal(size=100), dtype=torch.float32, device="cuda")
    gr = torch.tensor(rng.normal(size=100), dtype=torch.float32, device="cuda")
    m = torch.zeros(100, dtype=torch.float32, device="cuda")
    v = torch.zeros(100, dtype=torch.float32, device="cuda")
    p1 = p0.clone()
    assert lib.tbsg_adam(_p(p1), _p(gr), _p(m), _p(v), 100, 1e-2, 0.9, 0.999, 1e-8, 0.0, 1, None, st) == 0
    mh = 0.1 * gr.double() / 0.1
    vh = 0.001 * gr.double() ** 2 / 0.001
    want = p0.double() - 1e-2 * mh / (vh.sqrt() + 1e-8)
    assert (p1.double() - want).abs().max() <= 1e-6
    # global-norm clipping factor
    part = torch.empty(1024, dtype=torch.float32, device="cuda")
    cs = torch.empty(2, dtype=torch.float32, device="cuda")
    assert lib.tbsg_clip_scale(_p(gr), 100, 1.0, _p(part), _p(cs), st) == 0
    nrm = gr.double().norm().item()
    assert abs(cs[0].item() - nrm) <= 1e-6 * nrm and abs(cs[1].item() - min(1.0, 1.0 / nrm)) <= 1e-6


def _net_inputs(S, B, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(B, S, S, S, 16)).astype(np.float32)
    base = rng.uniform(0, 1, size=(B, S, S, S)).astype(np.float32)
    tgt = (base + 0.1 * rng.normal(size=base.shape)).astype(np.float32)
    return x, base, tgt


def _net_grads(seed=3, fused=True):
    S, B = 16, 2
    net = Surrogate(S, B, seed=seed)
    net.p[-(NFEAT + 1):].copy_(torch.linspace(-0.5, 0.5, NFEAT + 1))   # a non-zero head
    net.prep()
    x, base, tgt = _net_inputs(S, B, 1)
    xt = torch.tensor(x).cuda()
    bt, tt = torch.tensor(base).cuda(), torch.tensor(tgt).cuda()
    net.forward(xt, bt)
    loss = net.backward(tt, fused=fused).item()
    return net, xt, bt, tt, loss


def test_fused_backward_equals_unfused():
    """The backward pass with input gradients fused into the activation
    derivatives (the training path) gives the parameter gradients and the
    loss of the unfused pass bit for bit."""
    net, xt, bt, tt, loss = _net_grads(fused=True)
    g_fused = net.g.clone()
    loss2 = net.backward(tt, fused=False).item()
    assert loss2 == loss
    assert torch.equal(net.g, g_fused)


# (layer, input activation, output activation, gradient of the input or None, skip tensor or None)
WIRING = [("e0a", "x0", "e0a", None, None), ("e0b", "e0a", "e0", "e0a", None), ("e1a", "p1", "e1a", "p1", None),
          ("e1b", "e1a", "e1", "e1a", None), ("e2a", "p2", "e2a", "p2", None), ("e2b", "e2a", "e2", "e2a", None),
          ("e3a", "p3", "e3a", "p3", None), ("e3b", "e3a", "e3b", "e3a", None), ("e3c", "e3b", "e3", "e3b", None),
          ("d2a", "u2", "d2a", "u2", "e2"), ("d2b", "d2a", "d2", "d2a", None), ("d1a", "u1", "d1a", "u1", "e1"),
          ("d1b", "d1a", "d1", "d1a", None), ("d0a", "u0", "d0a", "u0", "e0"), ("d0b", "d0a", "d0", "d0a", None)]


def test_network_backward_wiring():
    """Every backward step of the network recomputed in float64 from the
    GPU's own activations and upstream gradients (exact up to FP32 sums)."""
    from trapbec_gb300.surrogate import SLOPE
    net, xt, bt, tt, loss = _net_grads(fused=False)   # every FP32 activation gradient in memory
    A = {k: v.double().cpu() for k, v in net.A.items()}
    G = {k: v.double().cpu() for k, v in net.G.items()}
    g = net.g.double().cpu()
    close = lambda a, b, tol=1e-5: (a - b).abs().max().item() <= tol * max(b.abs().max().item(), 1e-30)
    # head: dfeat = 2 (amp - target) / N * wh
    h0 = net.view["head"][0]
    wh, bh = net.p[h0:h0 + NFEAT].double().cpu(), net.p[h0 + NFEAT].double().cpu()
    amp = bt.double().cpu() + A["d0"] @ wh + bh
    dout = 2 * (amp - tt.double().cpu()) / amp.numel()
    assert close(G["d0"], dout[..., None] * wh)
    assert abs(loss - ((amp - tt.double().cpu()) ** 2).mean().item()) <= 1e-5 * loss
    skip_g = {}
    for name, xin, yout, gin, skip in WIRING:
        w0, b0, ci, co = net.view[name]
        # dz exactly as the kernel forms it: FP32 product, rounded to BF16
        gy, y = net.G[yout], net.A[yout]
        dyact = gy * torch.where(y.float() > 0, 1.0, SLOPE)
        dz = dyact.to(torch.bfloat16).double().cpu()
        if skip:
            skip_g[skip] = dyact.double().cpu()
        xr = A[xin].clone().requires_grad_(True)
        wr = net.wb[name].double().cpu().reshape(27, co, ci).clone().requires_grad_(True)
        br = torch.zeros(co, dtype=torch.float64, requires_grad=True)
        (nn_oracle.conv3(xr, wr, br) * dz).sum().backward()
        assert close(g[w0:b0].reshape(27, co, ci), wr.grad), name
        assert close(g[b0:b0 + co], br.grad), name
        if gin is not None:
            assert close(G[gin], xr.grad), (name, gin)
    # upsampling gradients and the skip + pooling sums
    up_sum = lambda t: t.reshape(t.shape[0], t.shape[1] // 2, 2, t.shape[2] // 2, 2, t.shape[3] // 2, 2,
                                 t.shape[4]).sum(dim=(2, 4, 6))
    assert close(G["d1"], up_sum(G["u0"]))
    assert close(G["d2"], up_sum(G["u1"]))
    assert close(G["e3"], up_sum(G["u2"]))
    for fine, coarse in (("e0", "p1"), ("e1", "p2"), ("e2", "p3")):
        assert close(G[fine], skip_g[fine] + nn_oracle.up2(G[coarse]) / 8), fine


def test_network_gradient_against_oracle():
    """End to end against the float64 oracle (BF16 drift bounds, see above)."""
    net, xt, bt, tt, loss = _net_grads()
    g = net.g.double().cpu().numpy()
    p = net.p.double().cpu().numpy()
    off = 0
    for name, ci, co in LAYERS:
        p[off:off + 27 * ci * co] = net.wb[name].double().cpu().numpy()
        off += 27 * ci * co + co
    xr = xt.to(torch.bfloat16).double().cpu().numpy()
    lref, gref = nn_oracle.loss_and_grad(p, xr, bt.double().cpu().numpy(), tt.double().cpu().numpy(), bf16=True)
    assert abs(loss - lref) <= 1e-3 * lref
    off = 0
    for name, ci, co in LAYERS:
        for a, b in ((off, off + 27 * ci * co), (off + 27 * ci * co, off + 27 * ci * co + co)):
            err = np.linalg.norm(g[a:b] - gref[a:b]) / np.linalg.norm(gref[a:b])
            assert err < 1.5e-1, (name, a == off, err)
        off += 27 * ci * co + co
    assert np.linalg.norm(g[off:] - gref[off:]) / np.linalg.norm(gref[off:]) < 1e-2


def test_training_reduces_loss():
    """A few hundred Adam steps on a small fixed set reduce the loss at least 5x."""
    S, B, N = 16, 2, 4
    net = Surrogate(S, B, seed=0)
    X, BASE, Y = [], [], []
    for i in range(N):
        x, base, tgt = _net_inputs(S, 1, 10 + i)
        X.append(x[0]); BASE.append(base[0]); Y.append(tgt[0])
    X = torch.tensor(np.stack(X)).cuda().to(torch.bfloat16)
    BASE = torch.tensor(np.stack(BASE)).cuda()
    Y = torch.tensor(np.stack(Y)).cuda()
    hist = train(net, X, BASE, Y, epochs=150, lr=2e-3, lr_min=1e-4)
    assert hist[-1] < hist[0] / 5, hist[::10]


def test_device_features_equal_host_features():
    """tbsg_features (the inference and training input path) writes the host
    recipe's channels rounded to BF16, bit for bit, and the FP32 base exactly."""
    import torch
    from trapbec_gb300 import units
    from trapbec_gb300.surrogate import features, features_device
    lib = abi.load()
    for prob, _ in units.ground_state_draws(3, 11, grids=(64, 96), precision=abi.FP32):
        f, base = features(prob)
        n = prob.n
        x = torch.empty(n + (NFEAT,), dtype=torch.bfloat16, device="cuda")
        b = torch.empty(n, dtype=torch.float32, device="cuda")
        features_device(lib, prob, x, b)
        torch.cuda.synchronize()
        want = torch.from_numpy(f).to(torch.bfloat16)
        assert torch.equal(x.cpu().view(torch.int16), want.view(torch.int16))
        assert np.array_equal(b.cpu().numpy().view(np.uint32), base.view(np.uint32))


def test_trained_weights_beat_thomas_fermi_guess():
    """What the trained network gains over the plain method, on held-out
    draws (the committed weights were trained on draws 0..TRAIN_DRAWS-1 of
    seed TRAIN_SEED): of the first eight held-out draws, those with
    Omega/omega_perp <= 0.5 (where the surrogate's guess is eligible), relaxed
    at 128^3 from both guesses to |d(E/N)| < 1e-10 per particle in trap
    units.  From the surrogate's guess the median step count is at least 3x
    smaller, the device time (counting the network's inference and the guess
    selector) is smaller, and the final state is the same (final energies
    within 1e-4 relative)."""
    import os
    from trapbec_gb300 import surrogate, units
    n0 = surrogate.TRAIN_DRAWS
    draws = units.ground_state_draws(n0 + 8, surrogate.TRAIN_SEED, grids=(128,), precision=abi.FP32)[n0:]
    draws = [d for d in draws if d[0].Omega <= 0.5 * d[0].omega[0]]
    assert len(draws) >= 3
    net = Surrogate(128, 2, seed=0)
    net.load(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                          "trapbec_gb300", "weights", "surrogate_128.npz"))
    r = surrogate.compare(net, draws, tol=1e-10, max_steps=20000, stop="per_particle")
    print({k: r[k] for k in ("nn_used", "steps_ratio_median", "wall_ratio_device",
                             "final_energy_rel_diff_max")}, r["tf"]["steps"], r["nn"]["steps"])
    assert r["nn_used"] == len(draws)
    assert all(r["nn"]["converged"])
    assert r["steps_ratio_median"] >= 3.0
    assert r["wall_ratio_device"] > 1.0
    assert r["same_end_state"] == len(draws) and r["final_energy_rel_diff_max"] <= 1e-4
