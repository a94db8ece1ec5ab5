"""Host-side pieces of the learned warm start (no GPU): the simulated objects
and probes of its training set and the C ABI's argument checks."""
import ctypes

import numpy as np

from ptychography_gb300 import _native
from ptychography_gb300 import warmstart as ws


def test_random_object_and_probe_ranges():
    rng = np.random.default_rng(0)
    O = ws.random_object(rng, 96)
    a, ph = np.abs(O), np.angle(O)
    assert O.shape == (96, 96)
    assert a.min() >= 0.5 - 1e-12 and a.max() <= 1.0 + 1e-12
    assert ph.min() >= -np.pi / 2 - 1e-12 and ph.max() <= np.pi / 2 + 1e-12
    P = ws.aperture_probe(64, 20, 3.0, 0.002)
    y, x = np.mgrid[:64, :64] - 32
    r = np.sqrt(x ** 2 + y ** 2)
    assert np.all(np.abs(P[r < 20]) > 0.999)
    assert np.all(P[r >= 20 + 9] == 0)
    np.testing.assert_allclose(np.angle(P[32, 32 + 5]), 0.002 * 25)


def test_network_layout():
    # six 3 x 3 convolutions, channels 32-128, (cos, sin) output
    # input: (Re, Im) of the back-projected object estimate
    assert len(ws.LAYERS) == 6 and ws.LAYERS[0][0] == 2 and ws.LAYERS[-1][1] == 2
    assert max(c for _, c, _, _ in ws.LAYERS) == 128
    assert [l for _, _, _, l in ws.LAYERS] == [0, 1, 2, 1, 0, 0]


def test_c_abi_rejects_bad_arguments_without_a_gpu():
    lib = _native.load()
    assert lib.pty_ws_gemm(0, 4, 4, None, 1, 1, None, 1, 1, None, 1, 1, 1, None, None) != 0
    assert lib.pty_ws_im2col(1, 0, 4, 4, None, None, None) != 0
    assert lib.pty_ws_pool2(1, 5, 4, 4, None, None, None) != 0        # odd side
    assert lib.pty_ws_act_bwd_scratch(0, 4) == -1
    assert lib.pty_ws_act_bwd_scratch(1000, 4) == 4 * 4                 # ceil(1000 / 256) blocks x C
    assert lib.pty_ws_adam(10, None, None, None, None, None, 1e-3, 0.9, 0.999, 1e-8, 1, None) != 0
    assert lib.pty_ws_prep_bp(1, 0, 8, None, None, 1, None, None) != 0
    one = ctypes.c_void_p(16)                                          # never dereferenced: rejected first
    assert lib.pty_ws_prep_bp(1, 8, 7, one, one, 1, one, None) != 0     # odd side with the sign correction
    assert b"even" in lib.pty_last_error()
    # the tensor-core training entries: shape rules and null arguments, checked on the host
    assert lib.pty_ws_wgrad_tc_scratch(2, 64, 64, 32, 64) > 0
    for args in ((1, 8, 64, 2, 32), (1, 8, 16, 32, 32), (1, 8, 96, 64, 32), (1, 8, 64, 32, 0)):
        assert lib.pty_ws_wgrad_tc_scratch(*args) == -1, args
    assert lib.pty_ws_wgrad_tc(1, 8, 64, 32, 32, None, one, one, one, 1 << 20, None) != 0
    assert lib.pty_ws_shift_transpose(1, 4, 7, 8, 3, one, one, None) != 0     # odd width
    assert lib.pty_ws_shift_transpose(1, 4, 8, 8, 2, one, one, None) != 0     # S must be 1 or 3
    assert lib.pty_ws_flip_weights(0, 4, one, one, None) != 0
    assert lib.pty_ws_conv3x3_tc_f32(1, 8, 8, 32, 32, None, one, one, None) != 0
    assert lib.pty_ws_align_phase(1, 8, 8, None, 16, 16, one, one, one, None) != 0
    assert lib.pty_ws_align_phase(1, 8, 8, one, 7, 16, one, one, one, None) != 0   # object smaller than a frame


def test_covering_frames_lights_every_pixel():
    """The warm start's frame subset: on a dense jittered raster (step 12 px,
    probe radius ~36 px at the network's sampling) it keeps well under half
    the frames, and every pixel the full scan lights gets at least 30 % of
    the best |P|^2 any frame gives it from some kept frame."""
    rng = np.random.default_rng(2)
    side, step, N = 32, 12, 128
    pos = np.arange(side) * step
    R = -np.stack(np.meshgrid(pos, pos, indexing="ij"), -1).reshape(-1, 2)
    R = R + rng.integers(-1, 2, R.shape)
    R = R - R.max(axis=0)
    P = ws.aperture_probe(N, 32, 4.0, 0.002)
    sel = ws.covering_frames(R, P)
    assert 0 < len(sel) < 0.45 * len(R)
    assert np.all(np.diff(sel) > 0)
    p2 = np.abs(P) ** 2
    U, V = N + int(R[:, 0].max() - R[:, 0].min()), N + int(R[:, 1].max() - R[:, 1].min())
    heat, best_all, best = np.zeros((U, V)), np.zeros((U, V)), np.zeros((U, V))
    for f, (r0, r1) in enumerate(R):
        w = (slice(-r0, -r0 + N), slice(-r1, -r1 + N))
        heat[w] += p2
        best_all[w] = np.maximum(best_all[w], p2)
        if f in set(sel.tolist()):
            best[w] = np.maximum(best[w], p2)
    lit = heat > 1e-2 * heat.max()
    assert np.all(best[lit] >= 0.3 * best_all[lit])


def _conv(x, w):
    """3 x 3 convolution (zero padding) of NHWC x with w[co][(ky*3+kx) C_in + ci]."""
    B, H, W, cin = x.shape
    co = w.shape[0]
    xp = np.zeros((B, H + 2, W + 2, cin))
    xp[:, 1:-1, 1:-1] = x
    wk = w.reshape(co, 3, 3, cin)
    return sum(np.einsum("bhwc,oc->bhwo", xp[:, ky:ky + H, kx:kx + W], wk[:, ky, kx])
               for ky in range(3) for kx in range(3))


def test_flipped_weights_give_the_input_gradient():
    """The identity the tensor-core training pass uses for its input
    gradients: dX = conv3x3(dZ, Wf) with Wf[ci][t C_out + co] = W[co][(8 - t)
    C_in + ci] (pty_ws_flip_weights), checked against the adjoint of the
    forward convolution, <conv(X, W), dZ> = <X, dX>, in float64."""
    rng = np.random.default_rng(0)
    B, H, W, cin, cout = 2, 6, 7, 3, 4
    x = rng.standard_normal((B, H, W, cin))
    w = rng.standard_normal((cout, 9 * cin))
    dz = rng.standard_normal((B, H, W, cout))
    wf = np.empty((cin, 9 * cout))
    for ci in range(cin):
        for t in range(9):
            for c in range(cout):
                wf[ci, t * cout + c] = w[c, (8 - t) * cin + ci]
    dx = _conv(dz, wf)
    np.testing.assert_allclose(np.sum(_conv(x, w) * dz), np.sum(x * dx), rtol=1e-12)
    # and element by element against the derivative of the forward sum
    for _ in range(5):
        b, i, j, c = (int(rng.integers(0, s)) for s in (B, H, W, cin))
        e = np.zeros_like(x)
        e[b, i, j, c] = 1.0
        np.testing.assert_allclose(np.sum(_conv(e, w) * dz), dx[b, i, j, c], rtol=1e-12, atol=1e-12)


def test_shifted_copies_give_the_weight_gradient():
    """The decomposition of pty_ws_wgrad_tc: dW[co][(ky*3+kx) C_in + ci] =
    sum_p dZ[p][co] XS[kx][ci][p shifted by ky - 1 rows], XS the layer input
    channel-major in three copies shifted by kx - 1 along x with zeros past
    the row ends (pty_ws_shift_transpose), rows outside the image zero (the
    TMA's fill), against the derivative of <conv(X, W), dZ> in W."""
    rng = np.random.default_rng(1)
    B, H, W, cin, cout = 2, 5, 6, 3, 2
    x = rng.standard_normal((B, H, W, cin))
    dz = rng.standard_normal((B, H, W, cout))
    xs = np.zeros((3, cin, B, H, W))
    for s in range(3):
        sh = s - 1
        for xx in range(W):
            if 0 <= xx + sh < W:
                xs[s, :, :, :, xx] = np.transpose(x[:, :, xx + sh, :], (2, 0, 1))
    dw = np.zeros((cout, 9 * cin))
    for ky in range(3):
        rows = np.zeros_like(xs)
        for y in range(H):
            if 0 <= y + ky - 1 < H:
                rows[:, :, :, y, :] = xs[:, :, :, y + ky - 1, :]
        for kx in range(3):
            dw[:, (ky * 3 + kx) * cin:(ky * 3 + kx + 1) * cin] = np.einsum(
                "bhwo,cbhw->oc", dz, rows[kx])
    w0 = rng.standard_normal((cout, 9 * cin))
    for _ in range(6):
        co, k = int(rng.integers(0, cout)), int(rng.integers(0, 9 * cin))
        e = np.zeros_like(w0)
        e[co, k] = 1.0
        np.testing.assert_allclose(np.sum(_conv(x, e) * dz), dw[co, k], rtol=1e-12, atol=1e-12)
