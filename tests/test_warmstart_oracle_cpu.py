"""Pins the warm start's CPU oracle (no GPU).

The warm start has no reference counterpart, so its oracle is pinned against
torch's float64 autograd of the same network: the forward pass, every weight
and bias gradient and the input gradient agree to float64 rounding.  Its BF16
rounding agrees bit for bit with torch's float -> bfloat16 conversion, its
Adam step with torch.optim.Adam, its target / exit-wave maps invert each
other, and its network input (the back-projected object estimate) has the
known answer of a flat object.  The sign identity that lets the device form
that back-projection from the reference-order kernel is checked here too.
"""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

from oracle import warmstart_oracle as wo
from ptychography_gb300 import warmstart as ws


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def test_layers_match_the_library():
    assert tuple(wo.LAYERS) == tuple(ws.LAYERS)


def test_bf16_round_matches_torch():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(20000) * 10.0 ** rng.integers(-30, 30, 20000),
                        [0.0, -0.0, 1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 65504.0, 1e-40]])
    x = x.astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).float().numpy().astype(np.float64)
    np.testing.assert_array_equal(wo.bf16_round(x), ref)
    # ties go to the even neighbour
    assert wo.bf16_round(np.float32(1.0 + 2.0 ** -8)) == 1.0
    assert wo.bf16_round(np.float32(1.0 + 3 * 2.0 ** -8)) == 1.0 + 2.0 ** -6


def torch_net(w, b, x):
    """The network in torch float64 (NCHW), weights [C_out][9 C_in] as the oracle's."""
    params = []
    for (cin, cout, _, _), wi, bi in zip(wo.LAYERS, w, b):
        wt = torch.from_numpy(np.asarray(wi, np.float64)).view(cout, 3, 3, cin).permute(0, 3, 1, 2)
        params.append((wt.contiguous().requires_grad_(True),
                       torch.from_numpy(np.asarray(bi, np.float64)).requires_grad_(True)))

    def conv(i, h, relu=True):
        z = F.conv2d(h, params[i][0], params[i][1], padding=1)
        return F.relu(z) if relu else z
    h1 = conv(0, x)
    h2 = conv(1, F.avg_pool2d(h1, 2))
    h3 = conv(2, F.avg_pool2d(h2, 2))
    h4 = conv(3, F.interpolate(h3, scale_factor=2, mode="nearest")) + h2
    h5 = conv(4, F.interpolate(h4, scale_factor=2, mode="nearest")) + h1
    return conv(5, h5, relu=False), params


@pytest.mark.parametrize("B,H,W", [(2, 8, 8), (1, 12, 16)])
def test_forward_and_gradients_match_torch_autograd(B, H, W):
    rng = np.random.default_rng(B * 100 + H + W)
    w, b = wo.init_weights(seed=3)
    b = [rng.standard_normal(bi.shape) * 0.1 for bi in b]
    x = rng.standard_normal((B, H, W, wo.LAYERS[0][0]))
    t = rng.standard_normal((B, H, W, 2))
    wgt = rng.random((B, H, W))
    wgt /= wgt.sum()
    y, cache = wo.forward(x, w, b)
    loss, dy = wo.loss_grad(y, t, wgt)
    gw, gb, dx = wo.backward(cache, dy)

    xt = torch.from_numpy(x).permute(0, 3, 1, 2).contiguous().requires_grad_(True)
    yt, params = torch_net(w, b, xt)
    lt = (torch.from_numpy(wgt)[:, None] * (yt - torch.from_numpy(t).permute(0, 3, 1, 2)) ** 2).sum()
    lt.backward()
    assert rel(y, yt.detach().permute(0, 2, 3, 1).numpy()) < 1e-12
    assert abs(loss - lt.item()) < 1e-12 * lt.item()
    for i, (cin, cout, _, _) in enumerate(wo.LAYERS):
        gw_ref = params[i][0].grad.permute(0, 2, 3, 1).reshape(cout, 9 * cin).numpy()
        assert rel(gw[i], gw_ref) < 1e-12, i
        assert rel(gb[i], params[i][1].grad.numpy()) < 1e-12, i
    assert rel(dx, xt.grad.permute(0, 2, 3, 1).numpy()) < 1e-12


def test_bf16_emulation_stays_close_to_float64():
    rng = np.random.default_rng(7)
    w, b = wo.init_weights(seed=1)
    x = rng.standard_normal((2, 16, 16, wo.LAYERS[0][0]))
    y64, c64 = wo.forward(x, w, b)
    y16, c16 = wo.forward(x, w, b, bf16=True)
    assert 0 < rel(y16, y64) < 3e-2
    dy = rng.standard_normal(y64.shape)
    g64, _, _ = wo.backward(c64, dy)
    g16, _, _ = wo.backward(c16, dy)
    for a, r in zip(g16, g64):                 # BF16 activations and gradients: a few %
        assert rel(a, r) < 1e-1


def test_adjoint_pairs():
    rng = np.random.default_rng(2)
    B, H, W, C = 2, 6, 8, 3
    x = rng.standard_normal((B, H, W, C))
    g = rng.standard_normal((B * H * W, 9 * C))
    assert np.isclose(np.sum(wo.im2col(x) * g), np.sum(x * wo.col2im(g, B, H, W, C)))
    p = rng.standard_normal((B, H // 2, W // 2, C))
    assert np.isclose(np.sum(wo.pool2(x) * p), np.sum(x * wo.pool2_bwd(p)))
    assert np.isclose(np.sum(wo.up2(p) * x), np.sum(p * wo.up2_bwd(x)))


def test_adam_matches_torch():
    rng = np.random.default_rng(4)
    w0 = rng.standard_normal(50)
    grads = [rng.standard_normal(50) for _ in range(5)]
    p = torch.from_numpy(w0.copy()).requires_grad_(True)
    opt = torch.optim.Adam([p], lr=3e-3, betas=(0.9, 0.999), eps=1e-8)
    w, m, v = w0.copy(), np.zeros(50), np.zeros(50)
    for k, g in enumerate(grads, 1):
        p.grad = torch.from_numpy(g.copy())
        opt.step()
        w, m, v = wo.adam(w, g, m, v, k, lr=3e-3)
    np.testing.assert_allclose(w, p.detach().numpy(), rtol=1e-13, atol=1e-15)


def test_data_maps():
    rng = np.random.default_rng(5)
    psi = rng.standard_normal((3, 8, 8)) + 1j * rng.standard_normal((3, 8, 8))
    P = rng.standard_normal((8, 8)) + 1j * rng.standard_normal((8, 8))
    for object_phase in (True, False):
        t, wgt = wo.targets(psi, P, object_phase, wscale=2.0)
        np.testing.assert_allclose(np.hypot(t[..., 0], t[..., 1]), 1.0)
        np.testing.assert_allclose(wgt, 2.0 * np.abs(P) ** 2 * np.ones((3, 1, 1)))
        # targets then exits restore |P| times the wave's phase
        np.testing.assert_allclose(wo.exits(t, P, object_phase), np.abs(P) * psi / np.abs(psi), atol=1e-12)


def test_bp_input_known_answers():
    """A flat object back-projects to the probe itself, so the input is
    |P|^2 / max|P|^2 (real); an empty frame gives zeros; the input scales out
    the object's amplitude."""
    P = ws.aperture_probe(32, 8, 2.0, 0.004)
    I1 = np.fft.fftshift(np.abs(np.fft.fft2(P)) ** 2)
    I = np.stack([I1, np.zeros_like(I1), 9.0 * I1])           # object 1, empty, object 3
    x = wo.bp_input(I, P)
    ref = np.abs(P) ** 2 / np.max(np.abs(P) ** 2)
    np.testing.assert_allclose(x[0, ..., 0], ref, atol=1e-12)
    np.testing.assert_allclose(x[0, ..., 1], 0.0, atol=1e-12)
    assert np.all(x[1] == 0.0)
    np.testing.assert_allclose(x[2], x[0], atol=1e-12)


@pytest.mark.parametrize("N0,N1", [(8, 8), (8, 12), (64, 64)])
def test_back_projection_sign_identity(N0, N1):
    """ifftn(fftshift(a) fftshift(phi)) = (-1)^(row + col) ifftn(a phi) for even
    sides: the reference-order back-projection kernel (amplitudes used in
    centred order) fed the shifted phasors gives the natural-order
    back-projection up to the checkerboard sign the input kernel removes."""
    rng = np.random.default_rng(N0 + N1)
    a = rng.random((2, N0, N1))
    phi = np.exp(2j * np.pi * rng.random((N0, N1)))
    lhs = np.fft.ifftn(np.fft.fftshift(a, axes=(-2, -1)) * np.fft.fftshift(phi), axes=(-2, -1))
    sign = (-1.0) ** np.add.outer(np.arange(N0), np.arange(N1))
    np.testing.assert_allclose(lhs, sign * np.fft.ifftn(a * phi, axes=(-2, -1)), atol=1e-12)
