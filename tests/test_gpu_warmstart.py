"""The warm-start network's kernels against plain PyTorch references on the CPU.

* the BF16 tensor-core GEMM in the three stride patterns a convolution uses
  (forward, dgrad, split-K wgrad) equals a float64 product of the same
  BF16-rounded operands to FP32-accumulation accuracy;
* im2col / col2im, pooling and upsampling pairs are exact adjoints;
* the whole forward pass and the weight / bias gradients of the backward
  pass match torch's float64 autograd of the same network within the
  rounding of BF16 activations and gradients (tolerances below);
* a few Adam steps on one batch reduce the loss.
"""
import ctypes

import numpy as np
import pytest
import torch
import torch.nn.functional as F

from ptychography_gb300 import _native
from ptychography_gb300.warmstart import LAYERS, WarmStartNet
from gpu_util import dev, stream

pytestmark = pytest.mark.gpu


def p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def bf(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev()).to(torch.bfloat16)


def gemm(M, N, K, A, sa, B, sb, splits=1):
    lib = _native.load()
    C = torch.zeros((M, N), dtype=torch.float32, device=dev())
    part = torch.empty((splits, M, N), dtype=torch.float32, device=dev()) if splits > 1 else None
    _native.check(lib.pty_ws_gemm(M, N, K, p(A), sa[0], sa[1], p(B), sb[0], sb[1], p(C), N, 1, splits,
                                  p(part), stream()))
    return C.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("M,N,K,splits", [(100, 70, 45, 1), (64, 64, 1000, 4), (3, 130, 4097, 7)])
def test_gemm_strides_match_fp64(M, N, K, splits):
    rng = np.random.default_rng(M + N + K)
    a = rng.standard_normal((M, K)).astype(np.float32)
    b = rng.standard_normal((K, N)).astype(np.float32)
    ab, bb = bf(a), bf(b)
    ar = ab.float().cpu().numpy().astype(np.float64)
    br = bb.float().cpu().numpy().astype(np.float64)
    ref = ar @ br
    tol = 1e-5 * np.sqrt(K)
    # A row-major, B row-major (k, n) -> sbk = N, sbn = 1
    c1 = gemm(M, N, K, ab, (K, 1), bb, (N, 1), splits)
    # A column-major (stored as its transpose), B column-major
    at, bt = bf(a.T), bf(b.T)
    c2 = gemm(M, N, K, at, (1, M), bt, (1, K), splits)
    for c in (c1, c2):
        assert np.linalg.norm(c - ref) / np.linalg.norm(ref) < tol


def test_adjoint_pairs():
    lib = _native.load()
    rng = np.random.default_rng(3)
    B, H, W, C = 2, 8, 12, 5
    x = rng.standard_normal((B, H, W, C)).astype(np.float32)
    xb = bf(x)
    col = torch.empty((B * H * W, 9 * C), dtype=torch.bfloat16, device=dev())
    _native.check(lib.pty_ws_im2col(B, H, W, C, p(xb), p(col), stream()))
    g = rng.standard_normal((B * H * W, 9 * C)).astype(np.float32)
    gd = torch.from_numpy(g).to(dev())
    dx = torch.empty((B, H, W, C), dtype=torch.float32, device=dev())
    _native.check(lib.pty_ws_col2im(B, H, W, C, p(gd), p(dx), stream()))
    xr = xb.float().cpu().numpy().astype(np.float64)
    lhs = float(np.sum(col.float().cpu().numpy().astype(np.float64) * g))
    rhs = float(np.sum(xr * dx.cpu().numpy()))
    assert abs(lhs - rhs) <= 1e-4 * abs(lhs)
    # pooling / upsampling against torch, and their adjoints
    xt = torch.from_numpy(xr).permute(0, 3, 1, 2)
    y = torch.empty((B, H // 2, W // 2, C), dtype=torch.bfloat16, device=dev())
    _native.check(lib.pty_ws_pool2(B, H, W, C, p(xb), p(y), stream()))
    ref = F.avg_pool2d(xt, 2).permute(0, 2, 3, 1).numpy()
    np.testing.assert_allclose(y.float().cpu().numpy(), ref, rtol=1e-2, atol=1e-2)
    u = torch.empty((B, 2 * H, 2 * W, C), dtype=torch.bfloat16, device=dev())
    _native.check(lib.pty_ws_up2(B, H, W, C, p(xb), p(u), stream()))
    ref = F.interpolate(xt, scale_factor=2, mode="nearest").permute(0, 2, 3, 1).numpy()
    np.testing.assert_array_equal(u.float().cpu().numpy(), ref.astype(np.float32))
    gu = torch.from_numpy(rng.standard_normal((B, 2 * H, 2 * W, C)).astype(np.float32)).to(dev())
    du = torch.empty((B, H, W, C), dtype=torch.float32, device=dev())
    _native.check(lib.pty_ws_up2_bwd(B, H, W, C, p(gu), p(du), stream()))
    ref = F.avg_pool2d(torch.from_numpy(gu.cpu().numpy().astype(np.float64)).permute(0, 3, 1, 2), 2) * 4
    np.testing.assert_allclose(du.cpu().numpy(), ref.permute(0, 2, 3, 1).numpy(), rtol=1e-5, atol=1e-5)


def torch_net(net, x):
    """The same network in float64 on the CPU (torch autograd), weights from net."""
    params = []
    for (cin, cout, _, _), w, b in zip(LAYERS, net.w, net.b):
        wt = torch.from_numpy(w.cpu().numpy().astype(np.float64)).view(cout, 3, 3, cin).permute(0, 3, 1, 2)
        wt = wt.contiguous().requires_grad_(True)
        bt = torch.from_numpy(b.cpu().numpy().astype(np.float64)).requires_grad_(True)
        params.append((wt, bt))

    def conv(i, h, relu=True):
        z = F.conv2d(h, params[i][0], params[i][1], padding=1)
        return F.relu(z) if relu else z
    h1 = conv(0, x)
    h2 = conv(1, F.avg_pool2d(h1, 2))
    h3 = conv(2, F.avg_pool2d(h2, 2))
    h4 = conv(3, F.interpolate(h3, scale_factor=2, mode="nearest")) + h2
    h5 = conv(4, F.interpolate(h4, scale_factor=2, mode="nearest")) + h1
    return conv(5, h5, relu=False), params


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def test_forward_and_gradients_match_torch_fp64():
    B, H, W = 2, 16, 16
    net = WarmStartNet(H, W, seed=1, device=dev())
    rng = np.random.default_rng(5)
    for b in net.b:                                  # non-zero biases
        b.copy_(torch.from_numpy(rng.standard_normal(b.shape).astype(np.float32) * 0.1))
    x = np.abs(rng.standard_normal((B, H, W, 1))).astype(np.float32)
    xb = bf(x)
    y = net.forward(xb)
    t = rng.standard_normal((B, H, W, 2)).astype(np.float32)
    wgt = rng.random((B, H, W)).astype(np.float32)
    wgt /= wgt.sum()
    td, wd = torch.from_numpy(t).to(dev()), torch.from_numpy(wgt).to(dev())
    parts, dy = net.loss_grad(y, td, wd)
    net.backward(dy)
    torch.cuda.synchronize()
    # reference on the BF16-rounded input and weights
    xr = torch.from_numpy(xb.float().cpu().numpy().astype(np.float64)).permute(0, 3, 1, 2)
    for w, wb in zip(net.w, net.wb):
        w.copy_(wb.float())
    yr, params = torch_net(net, xr)
    loss = (torch.from_numpy(wgt.astype(np.float64))[:, None] *
            (yr - torch.from_numpy(t.astype(np.float64)).permute(0, 3, 1, 2)) ** 2).sum()
    loss.backward()
    yg = y.cpu().numpy()
    # BF16 activations between layers: ~1 % per layer
    assert rel(yg, yr.detach().permute(0, 2, 3, 1).numpy()) < 5e-2
    assert abs(float(parts.sum().cpu()) - float(loss)) < 5e-2 * float(loss)
    for i, (cin, cout, _, _) in enumerate(LAYERS):
        gw_ref = params[i][0].grad.permute(0, 2, 3, 1).reshape(cout, 9 * cin).numpy()
        gb_ref = params[i][1].grad.numpy()
        gw = net.gw[i].cpu().numpy()
        gb = net.gb[i].cpu().numpy()
        assert rel(gw, gw_ref) < 8e-2, i
        assert rel(gb, gb_ref) < 8e-2, i
        cos = float(np.sum(gw * gw_ref) / (np.linalg.norm(gw) * np.linalg.norm(gw_ref)))
        assert cos > 0.995, i


def test_adam_steps_reduce_loss():
    B, H, W = 4, 16, 16
    net = WarmStartNet(H, W, seed=2, device=dev())
    rng = np.random.default_rng(9)
    x = bf(np.abs(rng.standard_normal((B, H, W, 1))))
    ang = rng.random((B, H, W)) * 2 * np.pi
    t = torch.from_numpy(np.stack([np.cos(ang), np.sin(ang)], -1).astype(np.float32)).to(dev())
    wgt = torch.full((B, H, W), 1.0 / (B * H * W), dtype=torch.float32, device=dev())
    losses = [float(net.train_step(x, t, wgt, lr=3e-3).sum().cpu()) for _ in range(30)]
    assert losses[-1] < 0.5 * losses[0]


def test_training_on_simulated_frames_learns_the_phase():
    """A short training run on simulated frames (random objects and probes)
    lowers the weighted phase error of held-out frames well below the
    untrained network's, and the stitched object of a held-out scan is a
    usable ERA start (the benchmark measures its time to NMSE 1e-3)."""
    from ptychography_gb300 import warmstart as ws
    N = 64
    net = ws.WarmStartNet(N, N, seed=0, device=dev())
    data = ws.make_training_set(net, 2048, seed=1, pad=32)
    held = ws.make_training_set(net, 256, seed=99, pad=32)

    def err(model):
        y = model.forward(held[0][:64])
        e = (y - held[1][:64]) ** 2
        return float((held[2][:64, ..., None] * e).sum())
    before = err(net)
    losses = ws.train(net, data, 400, batch=32, lr=3e-4)
    after = err(net)
    assert np.isfinite(losses).all()
    assert after < 0.6 * before and after < 1.0     # 1.0: predicting zero


def test_initial_object_feeds_era():
    """The public warm-start path: initial_object on host arrays, then ERA
    from it (known probe, object update) converges like ERA from ones."""
    import ptychography_gb300 as pty
    from ptychography_gb300 import warmstart as ws
    N = 64
    net = ws.WarmStartNet(N, N, seed=0, device=dev())
    ws.train(net, ws.make_training_set(net, 1024, seed=1, pad=32), 200, batch=32, lr=3e-4)
    rng = np.random.default_rng(4)
    O_true = ws.random_object(rng, 160)
    P = ws.aperture_probe(N, 16, 3.0, 0.004)
    pos = np.arange(8) * 12 + 4
    R = -np.stack(np.meshgrid(pos, pos, indexing="ij"), -1).reshape(-1, 2)
    ex = np.stack([O_true[-r0:-r0 + N, -r1:-r1 + N] * P for r0, r1 in R])
    I = np.fft.fftshift(np.abs(np.fft.fft2(ex)) ** 2, axes=(-2, -1)).astype(np.float32)
    O0 = ws.initial_object(net, I, R, P)
    assert O0.shape == (N + 84, N + 84) and np.isfinite(O0).all()
    O_a, info_a = pty.ERA(I, R.copy(), P, O0, 20, method=1)
    O_b, info_b = pty.ERA(I, R.copy(), P, None, 20, method=1)
    assert np.isfinite(O_a).all()
    assert info_a["eMod"][-1] < 2.0 * info_b["eMod"][-1]
