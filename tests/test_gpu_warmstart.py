"""The warm-start network's kernels against the CPU oracle and plain PyTorch
references on the CPU, and what the trained network gains.

* the BF16 tensor-core GEMM in the three stride patterns a convolution uses
  (forward, dgrad, split-K wgrad) equals a float64 product of the same
  BF16-rounded operands to FP32-accumulation accuracy;
* im2col / col2im, pooling and upsampling pairs are exact adjoints;
* the whole forward pass and the weight / bias gradients of the backward
  pass match torch's float64 autograd of the same network within the
  rounding of BF16 activations and gradients, and the CPU oracle
  (oracle/warmstart_oracle.py, run with the device's BF16 rounding points)
  to FP32-accumulation accuracy;
* Adam, the network input (back-projection), the targets and the predicted
  exit waves match the oracle;
* a few Adam steps on one batch reduce the loss; a short training run
  lowers the held-out phase error; the trained network's start beats ERA's
  start from ones before and after ERA iterations.
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
    x = rng.standard_normal((B, H, W, LAYERS[0][0])).astype(np.float32)
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
    x = bf(rng.standard_normal((B, H, W, LAYERS[0][0])))
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


def _scan(seed, N=64):
    """A held-out 8 x 8 scan (step 12) of a random object under the 64^2
    aperture probe: centred intensities, offsets, probe, the ground truth on
    the reconstruction grid and the illumination map."""
    from ptychography_gb300 import warmstart as ws
    rng = np.random.default_rng(seed)
    O_true = ws.random_object(rng, 160)
    P = ws.aperture_probe(N, 16, 3.0, 0.004)
    pos = np.arange(8) * 12 + 4
    R = -np.stack(np.meshgrid(pos, pos, indexing="ij"), -1).reshape(-1, 2)
    ex = np.stack([O_true[-r0:-r0 + N, -r1:-r1 + N] * P for r0, r1 in R])
    I = np.fft.fftshift(np.abs(np.fft.fft2(ex)) ** 2, axes=(-2, -1)).astype(np.float32)
    Rs = R - R.max(axis=0)
    U, V = N + int(np.ptp(Rs[:, 0])), N + int(np.ptp(Rs[:, 1]))
    heat = np.zeros((U, V))
    for r0, r1 in Rs:
        heat[-r0:-r0 + N, -r1:-r1 + N] += np.abs(P) ** 2
    off = -R.max(axis=0)
    return I, R, P, O_true[off[0]:off[0] + U, off[1]:off[1] + V], heat


def object_nmse(O, O_true, heat):
    """Object error over the illuminated region after removing the global complex scale."""
    m = heat > 1e-3 * heat.max()
    a, t = O[m].astype(np.complex128), O_true[m].astype(np.complex128)
    c = np.vdot(a, t) / np.vdot(a, a)
    return float(np.sum(np.abs(c * a - t) ** 2) / np.sum(np.abs(t) ** 2))


def test_trained_warm_start_gains_over_ones():
    """What the trained network gains over the method without it (ERA from an
    object of ones, era.py:480-486) on held-out scans: the object NMSE of the
    stitched start and after 5 ERA iterations (known probe), beside the same
    from the untrained network.  The public path: initial_object on host
    arrays, then pty.ERA from it."""
    import ptychography_gb300 as pty
    from ptychography_gb300 import warmstart as ws
    N = 64
    net = ws.WarmStartNet(N, N, seed=0, device=dev())
    scans = [_scan(s) for s in (4, 5)]
    untrained = [ws.initial_object(net, I, R, P) for I, R, P, _, _ in scans]
    ws.train(net, ws.make_training_set(net, 1024, seed=1, pad=32), 200, batch=32, lr=3e-4)
    for (I, R, P, Ot, heat), O_u in zip(scans, untrained):
        O0 = ws.initial_object(net, I, R, P)
        assert O0.shape == (N + 84, N + 84) and np.isfinite(O0).all()
        ones = np.ones_like(O0)
        O_w, info_w = pty.ERA(I, R.copy(), P, O0, 5, method=1)
        O_o, info_o = pty.ERA(I, R.copy(), P, None, 5, method=1)
        e = {"start_warm": object_nmse(O0, Ot, heat), "start_ones": object_nmse(ones, Ot, heat),
             "start_untrained": object_nmse(O_u, Ot, heat),
             "era5_warm": object_nmse(O_w, Ot, heat), "era5_ones": object_nmse(O_o, Ot, heat)}
        print("warm start vs ones (object NMSE):", {k: float("%.3g" % v) for k, v in e.items()})
        # measured on a GB300: start 0.085 / 0.055 against 0.19 / 0.146 from
        # ones (0.195 / 0.16 untrained); after 5 iterations 0.021 / 0.019
        # against 0.067 / 0.057
        assert np.isfinite(O_w).all()
        assert e["start_warm"] < 0.7 * e["start_ones"] and e["start_warm"] < 0.7 * e["start_untrained"]
        assert e["era5_warm"] < 0.6 * e["era5_ones"]


# ---------------------------------------------------------------- against the CPU oracle
def test_forward_and_gradients_match_the_oracle():
    """The device's forward pass, loss, output gradient and every weight and
    bias gradient against the CPU oracle run with the device's BF16 rounding
    points, so that only the FP32 accumulation order differs."""
    from oracle import warmstart_oracle as wo
    B, H, W = 2, 16, 16
    net = WarmStartNet(H, W, seed=4, device=dev())
    rng = np.random.default_rng(6)
    b_host = [(rng.standard_normal(b.shape) * 0.1).astype(np.float32) for b in net.b]
    for b, bh in zip(net.b, b_host):
        b.copy_(torch.from_numpy(bh))
    w_host = [w.cpu().numpy() for w in net.w]
    x = rng.standard_normal((B, H, W, LAYERS[0][0])).astype(np.float32)
    t = rng.standard_normal((B, H, W, 2)).astype(np.float32)
    wgt = rng.random((B, H, W)).astype(np.float32)
    wgt /= wgt.sum()
    y = net.forward(bf(x))
    parts, dy = net.loss_grad(y, torch.from_numpy(t).to(dev()), torch.from_numpy(wgt).to(dev()))
    net.backward(dy)
    torch.cuda.synchronize()
    yo, cache = wo.forward(x, w_host, b_host, bf16=True)
    lo, dyo = wo.loss_grad(y.cpu().numpy(), t, wgt)
    gwo, gbo, _ = wo.backward(cache, dy.cpu().numpy())
    errs = {"y": rel(y.cpu().numpy(), yo), "loss": abs(float(parts.sum().cpu()) - lo) / lo,
            "dy": rel(dy.cpu().numpy(), dyo)}
    for i in range(len(LAYERS)):
        errs["gw%d" % i] = rel(net.gw[i].cpu().numpy(), gwo[i])
        errs["gb%d" % i] = rel(net.gb[i].cpu().numpy(), gbo[i])
    print("warm-start network vs CPU oracle (relative):", {k: float("%.3g" % v) for k, v in errs.items()})
    # measured on a GB300: y 2e-7 to 3e-4 (single BF16 rounding flips), weight
    # gradients <= 8e-5, bias gradients <= 1.3e-5, loss 7e-8, dy 4e-8
    assert errs["loss"] < 1e-5 and errs["dy"] < 1e-6
    assert errs["y"] < 5e-3
    for i in range(len(LAYERS)):
        assert errs["gw%d" % i] < 2e-3 and errs["gb%d" % i] < 5e-4, i


def test_adam_matches_the_oracle():
    from oracle import warmstart_oracle as wo
    lib = _native.load()
    rng = np.random.default_rng(8)
    n = 1000
    w0 = rng.standard_normal(n).astype(np.float32)
    w = torch.from_numpy(w0).to(dev())
    wb = torch.empty(n, dtype=torch.bfloat16, device=dev())
    m = torch.zeros(n, dtype=torch.float32, device=dev())
    v = torch.zeros(n, dtype=torch.float32, device=dev())
    wo_, mo, vo = w0.astype(np.float64), np.zeros(n), np.zeros(n)
    for k in range(1, 6):
        g = (rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 1, n)).astype(np.float32)
        gd = torch.from_numpy(g).to(dev())
        _native.check(lib.pty_ws_adam(n, p(w), p(wb), p(gd), p(m), p(v), 3e-3, 0.9, 0.999, 1e-8, k, stream()))
        wo_, mo, vo = wo.adam(wo_, g, mo, vo, k, lr=3e-3)
    torch.cuda.synchronize()
    np.testing.assert_allclose(w.cpu().numpy(), wo_, rtol=0, atol=1e-6)
    np.testing.assert_allclose(m.cpu().numpy(), mo, rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(v.cpu().numpy(), vo, rtol=1e-4, atol=1e-14)
    np.testing.assert_array_equal(wb.float().cpu().numpy(), wo.bf16_round(w.cpu().numpy()))


def test_data_maps_match_the_oracle():
    """Network input (the back-projected object estimate, formed through a
    plan from centred intensities), training targets and predicted exit waves."""
    from oracle import warmstart_oracle as wo
    from ptychography_gb300 import warmstart as ws
    lib = _native.load()
    rng = np.random.default_rng(10)
    nf, N = 3, 64
    net = WarmStartNet(N, N, seed=0, device=dev())
    Pn = ws.aperture_probe(N, 16, 3.0, 0.004)
    O = ws.random_object(rng, N)
    I = np.stack([np.fft.fftshift(np.abs(np.fft.fft2(Pn * np.roll(O, (7 * i, 3 * i), (0, 1))) * s) ** 2)
                  for i, s in enumerate((1.0, 0.0, 30.0))]).astype(np.float32)       # frame 1 empty
    plan = ws._FramePlan(nf, N, N, N, np.zeros((nf, 2), np.int64))
    try:
        P_d = torch.from_numpy(Pn.astype(np.complex64)).to(dev())
        I_d = torch.from_numpy(I).to(dev())
        x = net.input_from_intensities(plan.h, I_d, P_d, ws.probe_phasors(Pn, dev()))
        torch.cuda.synchronize()
    finally:
        plan.close()
    xo = wo.bp_input(I, Pn)
    xg = x.float().cpu().numpy()
    np.testing.assert_allclose(xg, xo, rtol=2.0 ** -7, atol=1e-4 * np.abs(xo).max())
    assert np.all(xg[1] == 0)
    H, W = 32, 48
    psi = (rng.standard_normal((nf, H, W)) + 1j * rng.standard_normal((nf, H, W))).astype(np.complex64)
    psi[1, 0, :5] = 0
    P = (rng.standard_normal((H, W)) + 1j * rng.standard_normal((H, W))).astype(np.complex64)
    psi_d, P_d = torch.from_numpy(psi).to(dev()), torch.from_numpy(P).to(dev())
    for object_phase in (1, 0):
        tgt = torch.empty((nf, H, W, 2), dtype=torch.float32, device=dev())
        wgt = torch.empty((nf, H, W), dtype=torch.float32, device=dev())
        _native.check(lib.pty_ws_targets(nf, H * W, p(psi_d), p(P_d), object_phase, 0.5, p(tgt), p(wgt), stream()))
        to, wgo = wo.targets(psi, P, bool(object_phase), 0.5)
        np.testing.assert_allclose(tgt.cpu().numpy(), to, rtol=0, atol=2e-6)
        np.testing.assert_allclose(wgt.cpu().numpy(), wgo, rtol=2e-6, atol=0)
        y = torch.from_numpy(rng.standard_normal((nf, H, W, 2)).astype(np.float32)).to(dev())
        y[0, 0, :4] = 0.0                                # a zero prediction reads as phase 0
        out = torch.empty((nf, H, W), dtype=torch.complex64, device=dev())
        _native.check(lib.pty_ws_exits(nf, H * W, p(y), p(P_d), object_phase, p(out), stream()))
        eo = wo.exits(y.cpu().numpy(), P, bool(object_phase))
        np.testing.assert_allclose(out.cpu().numpy(), eo, rtol=0, atol=2e-6 * np.abs(P).max())
