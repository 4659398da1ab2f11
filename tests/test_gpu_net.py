"""Learned preconditioner: each kernel of the network against PyTorch CPU
float32 convolutions on the same bf16 values, the whole network's output and
parameter gradients against the CPU reference network (oracle/net_ref.py),
one fused Adam step against the textbook formula, and what training gains
for CG."""

import math

import pytest
import torch
import torch.nn.functional as F

from adrt_gb300 import _lib

pytestmark = pytest.mark.gpu

BF = torch.bfloat16


def lib():
    return _lib.load()


def stream():
    return torch.cuda.current_stream().cuda_stream


def nhwc(B, h, w, c, seed, scale=1.0):
    g = torch.Generator().manual_seed(seed)
    return (torch.randn((B, h, w, c), generator=g) * scale).to(BF)


def to_nchw(t):
    return t.float().permute(0, 3, 1, 2)


def to_nhwc(t):
    return t.permute(0, 2, 3, 1).contiguous()


def torch_weight(w9, ci, co):
    """[9][co][ci] -> (co, ci, 3, 3)."""
    return w9.float().reshape(3, 3, co, ci).permute(2, 3, 0, 1)


def rel(a, b):
    return float((a.float() - b.float()).norm() / b.float().norm().clamp_min(1e-30))


CONV_CASES = [
    # (c_in, c_out, h, w)
    (32, 32, 128, 128),
    (32, 64, 64, 64),
    (64, 32, 256, 256),
    (64, 128, 32, 32),
    (128, 256, 16, 16),
    (256, 128, 32, 32),
    (256, 256, 16, 16),
    (128, 64, 128, 128),
]


@pytest.mark.parametrize("ci,co,h,w", CONV_CASES)
def test_conv3x3_forward(ci, co, h, w):
    B = 2
    x = nhwc(B, h, w, ci, 1)
    wt = (torch.randn((9, co, ci), generator=torch.Generator().manual_seed(2)) / math.sqrt(9 * ci)).to(BF)
    bias = torch.randn(co, generator=torch.Generator().manual_seed(3))
    add = nhwc(B, h, w, co, 4, 0.5)
    want = F.conv2d(to_nchw(x), torch_weight(wt, ci, co), bias, padding=1) + to_nchw(add)
    want = to_nhwc(F.relu(want))
    xd, wd, bd, ad = x.cuda(), wt.cuda(), bias.cuda(), add.cuda()
    out = torch.empty((B, h, w, co), dtype=BF, device="cuda")
    rc = lib().adrtnet_conv3x3(xd.data_ptr(), ci, wd.data_ptr(), co, bd.data_ptr(), ad.data_ptr(), None, 1,
                               out.data_ptr(), B, h, w, stream())
    _lib.check(rc, "conv3x3")
    torch.cuda.synchronize()
    _lib.check(lib().adrtnet_status(stream()), "status")
    got = out.cpu().float()
    assert rel(got, want) < 8e-3, rel(got, want)


@pytest.mark.parametrize("ci,co,h,w", CONV_CASES[:5])
def test_conv3x3_input_gradient(ci, co, h, w):
    """dx = conv with the flipped, transposed weights, masked."""
    B = 2
    x = nhwc(B, h, w, ci, 5)
    w9 = (torch.randn((9, co, ci), generator=torch.Generator().manual_seed(6)) / math.sqrt(9 * ci)).to(BF)
    gy = nhwc(B, h, w, co, 7)
    mask = nhwc(B, h, w, ci, 8)
    xr = to_nchw(x).requires_grad_(True)
    y = F.conv2d(xr, torch_weight(w9, ci, co), padding=1)
    y.backward(to_nchw(gy))
    want = to_nhwc(xr.grad * (to_nchw(mask) > 0))
    wflip = torch.empty((9, ci, co), dtype=BF)
    for t in range(9):
        wflip[8 - t] = w9[t].t()
    gd, wd, md = gy.cuda(), wflip.cuda(), mask.cuda()
    out = torch.empty((B, h, w, ci), dtype=BF, device="cuda")
    rc = lib().adrtnet_conv3x3(gd.data_ptr(), co, wd.data_ptr(), ci, None, None, md.data_ptr(), 0,
                               out.data_ptr(), B, h, w, stream())
    _lib.check(rc, "conv3x3 dgrad")
    torch.cuda.synchronize()
    got = out.cpu().float()
    assert rel(got, want) < 8e-3, rel(got, want)


@pytest.mark.parametrize("ci,co,h,w", CONV_CASES)
def test_conv3x3_weight_gradient(ci, co, h, w):
    B = 2
    x = nhwc(B, h, w, ci, 9)
    gy = nhwc(B, h, w, co, 10)
    wz = torch.zeros((co, ci, 3, 3), requires_grad=True)
    y = F.conv2d(to_nchw(x), wz, padding=1)
    y.backward(to_nchw(gy))
    want = wz.grad.permute(2, 3, 0, 1).reshape(9, co, ci)
    xd, gd = x.cuda(), gy.cuda()
    dw = torch.full((9, co, ci), 0.25, device="cuda")  # accumulates onto existing values
    rc = lib().adrtnet_conv3x3_wgrad(xd.data_ptr(), ci, gd.data_ptr(), co, dw.data_ptr(), B, h, w, stream())
    _lib.check(rc, "wgrad")
    torch.cuda.synchronize()
    _lib.check(lib().adrtnet_status(stream()), "status")
    got = dw.cpu() - 0.25
    assert rel(got, want) < 1e-4, rel(got, want)


def test_conv3x3_rejects_bad_shapes():
    t = torch.empty(16, dtype=BF, device="cuda")
    p = t.data_ptr()
    L = lib()
    assert L.adrtnet_conv3x3(p, 48, p, 32, None, None, None, 1, p, 1, 16, 16, stream()) == _lib.ERR_SHAPE
    assert L.adrtnet_conv3x3(p, 32, p, 32, None, None, None, 1, p, 1, 8, 8, stream()) == _lib.ERR_SHAPE
    assert L.adrtnet_conv3x3(None, 32, p, 32, None, None, None, 1, p, 1, 16, 16, stream()) == _lib.ERR_NULL
    assert L.adrtnet_conv3x3_wgrad(p, 32, p, 32, p, 1, 4, 8, stream()) == _lib.ERR_SHAPE


def test_small_kernels():
    B, h, w = 2, 32, 64
    L = lib()
    g = torch.Generator().manual_seed(11)
    u = torch.randn((B, h, w), generator=g)
    w_in = torch.randn((9, 32), generator=g) / 3
    b_in = torch.randn(32, generator=g) * 0.1
    # Device copies are held in variables: a temporary freed before the
    # launch could be reused by the next copy.
    ud, w_ind, b_ind = u.cuda(), w_in.cuda(), b_in.cuda()
    a0 = torch.empty((B, h, w, 32), dtype=BF, device="cuda")
    _lib.check(L.adrtnet_conv_in(ud.data_ptr(), w_ind.data_ptr(), b_ind.data_ptr(), a0.data_ptr(), B, h, w,
                                 stream()), "conv_in")
    want = F.relu(F.conv2d(u[:, None], w_in.reshape(3, 3, 32).permute(2, 0, 1)[:, None], b_in, padding=1))
    assert rel(a0.cpu().float(), to_nhwc(want)) < 5e-3

    f = nhwc(B, h, w, 32, 12)
    w_out = torch.randn((9, 32), generator=g) / 17
    b_out = torch.randn(1, generator=g)
    out = torch.empty((B, h, w), device="cuda")
    fd, w_outd, b_outd = f.cuda(), w_out.cuda(), b_out.cuda()
    _lib.check(L.adrtnet_conv_out(fd.data_ptr(), w_outd.data_ptr(), b_outd.data_ptr(), out.data_ptr(), B, h, w,
                                  stream()), "conv_out")
    wt = w_out.reshape(3, 3, 32).permute(2, 0, 1)[None]
    fr = to_nchw(f).requires_grad_(True)
    wr = wt.clone().requires_grad_(True)
    br = b_out.clone().requires_grad_(True)
    y = F.conv2d(fr, wr, br, padding=1)[:, 0]
    assert rel(out.cpu(), y.detach()) < 1e-5
    gout = torch.randn((B, h, w), generator=g)
    y.backward(gout)
    goutd = gout.cuda()
    dx = torch.empty((B, h, w, 32), dtype=BF, device="cuda")
    dw = torch.zeros((9, 32), device="cuda")
    db = torch.zeros(1, device="cuda")
    _lib.check(L.adrtnet_conv_out_bwd(goutd.data_ptr(), w_outd.data_ptr(), fd.data_ptr(), dx.data_ptr(),
                                      dw.data_ptr(), db.data_ptr(), B, h, w, stream()), "conv_out_bwd")
    assert rel(dx.cpu().float(), to_nhwc(fr.grad * (to_nchw(f) > 0))) < 5e-3
    assert rel(dw.cpu(), wr.grad[0].permute(1, 2, 0).reshape(9, 32)) < 1e-4
    assert rel(db.cpu(), br.grad) < 1e-4

    # first-layer weight gradient
    ga = nhwc(B, h, w, 32, 13)
    gad = ga.cuda()
    wr = w_in.reshape(3, 3, 32).permute(2, 0, 1)[:, None].clone().requires_grad_(True)
    br = b_in.clone().requires_grad_(True)
    F.conv2d(u[:, None], wr, br, padding=1).backward(to_nchw(ga))
    dw = torch.zeros((9, 32), device="cuda")
    db = torch.zeros(32, device="cuda")
    _lib.check(L.adrtnet_conv_in_wgrad(ud.data_ptr(), gad.data_ptr(), dw.data_ptr(), db.data_ptr(), B, h, w,
                                       stream()), "conv_in_wgrad")
    assert rel(dw.cpu(), wr.grad[:, 0].permute(1, 2, 0).reshape(9, 32)) < 1e-4
    assert rel(db.cpu(), br.grad) < 1e-4

    # pooling, upsampling and their backward passes; bias gradient
    x = nhwc(B, h, w, 64, 14)
    xd = x.cuda()
    p = torch.empty((B, h // 2, w // 2, 64), dtype=BF, device="cuda")
    _lib.check(L.adrtnet_pool2(xd.data_ptr(), p.data_ptr(), B, h, w, 64, stream()), "pool2")
    assert rel(p.cpu().float(), to_nhwc(F.avg_pool2d(to_nchw(x), 2))) < 5e-3
    up = torch.empty((B, 2 * h, 2 * w, 64), dtype=BF, device="cuda")
    _lib.check(L.adrtnet_up2(xd.data_ptr(), up.data_ptr(), B, h, w, 64, stream()), "up2")
    assert torch.equal(up.cpu(), to_nhwc(F.interpolate(to_nchw(x), scale_factor=2, mode="nearest")).to(BF))
    gl = nhwc(B, h // 2, w // 2, 64, 15)
    skip = nhwc(B, h, w, 64, 16)
    mask = nhwc(B, h, w, 64, 17)
    gld, skipd, maskd = gl.cuda(), skip.cuda(), mask.cuda()
    o = torch.empty((B, h, w, 64), dtype=BF, device="cuda")
    _lib.check(L.adrtnet_pool2_bwd(gld.data_ptr(), skipd.data_ptr(), maskd.data_ptr(), o.data_ptr(), B, h, w, 64,
                                   stream()), "pool2_bwd")
    want = (to_nchw(skip) + F.interpolate(to_nchw(gl), scale_factor=2, mode="nearest") / 4) * (to_nchw(mask) > 0)
    assert rel(o.cpu().float(), to_nhwc(want)) < 5e-3
    gh = nhwc(B, 2 * h, 2 * w, 64, 18)
    ghd = gh.cuda()
    o = torch.empty((B, h, w, 64), dtype=BF, device="cuda")
    _lib.check(L.adrtnet_up2_bwd(ghd.data_ptr(), maskd.data_ptr(), o.data_ptr(), B, h, w, 64, stream()), "up2_bwd")
    want = F.avg_pool2d(to_nchw(gh), 2) * 4 * (to_nchw(mask) > 0)
    assert rel(o.cpu().float(), to_nhwc(want)) < 5e-3
    db = torch.zeros(64, device="cuda")
    _lib.check(L.adrtnet_bias_grad(xd.data_ptr(), db.data_ptr(), B * h * w, 64, stream()), "bias_grad")
    assert rel(db.cpu(), x.float().sum(dim=(0, 1, 2))) < 1e-4


@pytest.fixture(scope="module")
def small_net():
    from adrt_gb300.learned import PreconditionerNet

    net = PreconditionerNet("cuda", seed=3)
    # Non-zero biases so that every bias path is exercised.
    g = torch.Generator().manual_seed(4)
    for name in list(net.offsets):
        if name.endswith("_b"):
            v = net.view(name)
            v.copy_(torch.randn(v.shape, generator=g).cuda() * 0.05)
    net.refresh_weights()
    return net


def test_network_matches_cpu_reference(small_net):
    from oracle import net_ref

    net = small_net
    B, n = 2, 128
    g = torch.Generator().manual_seed(21)
    u = torch.rand((B, n, n), generator=g)
    target = torch.rand((B, n, n), generator=g)
    # Reference on the bf16-rounded tensor-core weights the kernels read.
    p_ref = net.params.detach().cpu().clone()
    offs, total = net_ref.offsets()
    assert total == net.n_params
    for name, (o, c, shape) in offs.items():
        if shape is not None:
            p_ref[o:o + c] = p_ref[o:o + c].to(BF).float()
    out_ref, loss_ref, grad_ref = net_ref.loss_and_grads(p_ref, u, target)

    ud = u.cuda()
    net.grads.zero_()
    out = net.forward(ud)
    assert rel(out.cpu(), out_ref) < 3e-2, rel(out.cpu(), out_ref)
    gout, loss = net.loss_and_grad(out, target.cuda())
    net.backward(ud, gout)
    torch.cuda.synchronize()
    net.check_status()
    assert abs(float(loss) - loss_ref) / loss_ref < 3e-2
    grads = net.grads.cpu()
    for name, (o, c, shape) in offs.items():
        e = rel(grads[o:o + c], grad_ref[o:o + c])
        assert e < 8e-2, (name, e)
    # whole gradient direction
    cos = float(torch.dot(grads, grad_ref) / (grads.norm() * grad_ref.norm()))
    assert cos > 0.998, cos


def test_adam_step_and_weight_copies(small_net):
    net = small_net
    p0 = net.params.detach().cpu().clone()
    g = torch.randn(net.n_params, generator=torch.Generator().manual_seed(5))
    net.grads.copy_(g.cuda())
    net.m.zero_()
    net.v.zero_()
    net.step_count.zero_()
    net.adam(lr=1e-2)
    torch.cuda.synchronize()
    m = 0.1 * g
    v = 0.001 * g * g
    want = p0 - 1e-2 * (m / 0.1) / (torch.sqrt(v / 0.001) + 1e-8)
    assert rel(net.params.cpu(), want) < 1e-6
    # bf16 copies: forward layout and the flipped/transposed layout.
    for name, ci, co in [("enc1a", 32, 64), ("dec2a", 256, 128)]:
        w = net.view(name + "_w").cpu().reshape(9, co, ci)
        assert torch.equal(net.wt(name).cpu().reshape(9, co, ci), w.to(BF))
        wt = net.wt(name, transposed=True).cpu().reshape(9, ci, co)
        for t in range(9):
            assert torch.equal(wt[8 - t], w[t].t().to(BF))


def test_training_gains_over_plain_cg():
    """A short training run on 128 x 128 phantoms: the learned start needs
    fewer CG iterations than the zero start on held-out data, and every
    solve still reaches the tolerance."""
    from adrt_gb300 import cg as cgmod
    from adrt_gb300 import learned

    n = 128
    b_tr, x_tr = learned.training_pairs(512, n, seed=100, tol=1e-5)
    net = learned.PreconditionerNet("cuda", seed=0)
    log = learned.train(net, b_tr, x_tr, epochs=12, batch=16, lr=1e-3)
    assert log.losses[-1] < log.losses[0]
    b_te, _ = learned.training_pairs(64, n, seed=50_000, tol=1e-5)
    plain = cgmod.cg(b_te, tol=1e-4, max_iters=500)
    lrn = learned.learned_cg(net, b_te, tol=1e-4, max_iters=500)
    assert (lrn.normal_residual <= 1.5e-4).all()
    assert float(lrn.iterations.float().mean()) < float(plain.iterations.float().mean())
