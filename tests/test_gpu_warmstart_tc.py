"""The warm-start network's tensor-core convolution (pty_ws_conv3x3_tc:
tcgen05 MMAs accumulating in tensor memory, TMA-staged operands, bias /
activation / skip fused) against a float64 reference of the same BF16
operands, against the im2col + mma.sync GEMM path, and as the bulk of the
network's inference pass.

Tolerances: the products of BF16 operands are exact in FP32, so the sums
differ from float64 only by FP32 accumulation rounding (~1e-6 relative); the
BF16 output rounding adds up to 2^-9 relative per element, i.e. ~1.6e-3
norm-wise.  Against the im2col path (the same operands, another FP32
summation order) elements may differ by one BF16 rounding step.
"""
import ctypes

import numpy as np
import pytest
import torch

from gpu_util import dev, stream
from ptychography_gb300 import _native
from ptychography_gb300.warmstart import LAYERS, WarmStartNet

pytestmark = pytest.mark.gpu


def p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def conv_ref(x, w, b, relu, skip):
    """float64 3 x 3 convolution (zero padding) of NHWC x with w[co][(ky*3+kx) C + ci]."""
    B, H, W, C = x.shape
    co = w.shape[0]
    xp = np.zeros((B, H + 2, W + 2, C))
    xp[:, 1:-1, 1:-1] = x
    wk = w.reshape(co, 3, 3, C)
    z = np.zeros((B, H, W, co))
    for ky in range(3):
        for kx in range(3):
            z += np.einsum("bhwc,oc->bhwo", xp[:, ky:ky + H, kx:kx + W], wk[:, ky, kx])
    z += b
    if relu:
        z = np.maximum(z, 0)
    z = z.astype(np.float32)
    z = torch.from_numpy(z).to(torch.bfloat16).float().numpy().astype(np.float64)
    if skip is not None:
        z = torch.from_numpy((z + skip).astype(np.float32)).to(torch.bfloat16).float().numpy()
    return z


def bf16(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev()).to(torch.bfloat16)


def status_ok():
    t = ctypes.c_int32(-1)
    _native.check(_native.load().pty_timeout_status(ctypes.byref(t)))
    return t.value == 0


# (B, H, W, C_in, C_out, relu, skip): the network's layers 1-4 at 128^2 frames,
# plus a 256-wide image (two tiles per row) and a 32-channel-in layer with
# skip; one-row tiles of 64 input channels and C_out <= 64 take the halo
# staging (layer 4, the 256-wide 64 -> 64 case with halos across tiles, and a
# 3-row image whose every tile meets the top or bottom edge)
CASES = [(2, 64, 64, 32, 64, True, False), (2, 32, 32, 64, 128, True, False),
         (2, 64, 64, 128, 64, True, True), (2, 128, 128, 64, 32, True, True),
         (1, 8, 256, 64, 96, False, False), (3, 16, 16, 32, 32, True, True),
         (1, 4, 256, 64, 64, True, True), (2, 3, 128, 64, 32, False, False)]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:5])))
def test_conv_tc_matches_fp64_and_im2col_path(case):
    B, H, W, cin, cout, relu, has_skip = case
    lib = _native.load()
    rng = np.random.default_rng(B * H + W + cin + cout)
    x = rng.standard_normal((B, H, W, cin)).astype(np.float32)
    w = (rng.standard_normal((cout, 9 * cin)) * np.sqrt(2.0 / (9 * cin))).astype(np.float32)
    b = (0.1 * rng.standard_normal(cout)).astype(np.float32)
    sk = rng.standard_normal((B, H, W, cout)).astype(np.float32) if has_skip else None
    xd, wd = bf16(x), bf16(w)
    bd = torch.from_numpy(b).to(dev())
    skd = bf16(sk) if has_skip else None
    out = torch.empty((B, H, W, cout), dtype=torch.bfloat16, device=dev())
    _native.check(lib.pty_ws_conv3x3_tc(B, H, W, cin, cout, p(xd), p(wd), p(bd), int(relu), p(skd),
                                        p(out), None, stream()))
    assert status_ok()
    got = out.float().cpu().numpy().astype(np.float64)
    xr = xd.float().cpu().numpy().astype(np.float64)
    wr = wd.float().cpu().numpy().astype(np.float64)
    skr = skd.float().cpu().numpy().astype(np.float64) if has_skip else None
    ref = conv_ref(xr, wr, b.astype(np.float64), relu, skr)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 3e-3
    # the im2col + GEMM + bias/activation path on the same operands
    P, K = B * H * W, 9 * cin
    col = torch.empty((P, K), dtype=torch.bfloat16, device=dev())
    _native.check(lib.pty_ws_im2col(B, H, W, cin, p(xd), p(col), stream()))
    Z = torch.empty((P, cout), dtype=torch.float32, device=dev())
    _native.check(lib.pty_ws_gemm(P, cout, K, p(col), K, 1, p(wd), 1, K, p(Z), cout, 1, 1, None, stream()))
    a = torch.empty((B, H, W, cout), dtype=torch.bfloat16, device=dev())
    o2 = torch.empty((B, H, W, cout), dtype=torch.bfloat16, device=dev()) if has_skip else None
    _native.check(lib.pty_ws_bias_act(P, cout, p(Z), p(bd), int(relu), p(skd), p(a),
                                      p(o2) if has_skip else None, None, stream()))
    old = (o2 if has_skip else a).float().cpu().numpy().astype(np.float64)
    d = np.abs(got - old)
    assert np.linalg.norm(d) / np.linalg.norm(old) < 2e-3
    # elementwise: within two BF16 rounding steps of the magnitude (skip adds a second rounding)
    assert np.all(d <= 2 ** -6 * np.maximum(np.abs(old), np.abs(got)) + 1e-6)


def dgrad_ref(dz, w):
    """float64 input gradient of the 3 x 3 convolution: dX[b, y, x, ci] =
    sum_{ky, kx, co} dZ[b, y - ky + 1, x - kx + 1, co] w[co][(ky*3+kx) C_in + ci]."""
    B, H, W, co = dz.shape
    cin = w.shape[1] // 9
    dzp = np.zeros((B, H + 2, W + 2, co))
    dzp[:, 1:-1, 1:-1] = dz
    wk = w.reshape(co, 3, 3, cin)
    dx = np.zeros((B, H, W, cin))
    for ky in range(3):
        for kx in range(3):
            dx += np.einsum("bhwo,oc->bhwc", dzp[:, 2 - ky:2 - ky + H, 2 - kx:2 - kx + W], wk[:, ky, kx])
    return dx


# (B, H, W, C_in, C_out) of the forward layer whose input gradient is taken:
# the network's layers 1-5 at 128^2 frames (layer 5, C_out 2, on the direct kernel)
DGRAD_CASES = [(2, 64, 64, 32, 64), (2, 32, 32, 64, 128), (2, 64, 64, 128, 64), (2, 128, 128, 64, 32),
               (2, 128, 128, 32, 2)]


@pytest.mark.parametrize("case", DGRAD_CASES, ids=lambda c: "x".join(map(str, c)))
def test_input_gradient_convolution_matches_fp64(case):
    """dX = conv3x3(dZ, Wf), Wf from pty_ws_flip_weights, on the tensor-core
    kernel's FP32 output mode (the direct kernel for a 2-channel dZ), against
    the float64 adjoint of the forward convolution on the same BF16 operands:
    the products are exact in FP32, so within 1e-5 norm-wise."""
    B, H, W, cin, cout = case
    lib = _native.load()
    rng = np.random.default_rng(B + H + cin + cout)
    dz = bf16(rng.standard_normal((B, H, W, cout)))
    wd = bf16(rng.standard_normal((cout, 9 * cin)) * np.sqrt(2.0 / (9 * cin)))
    wf = torch.empty((cin, 9 * cout), dtype=torch.bfloat16, device=dev())
    _native.check(lib.pty_ws_flip_weights(cin, cout, p(wd), p(wf), stream()))
    dx = torch.empty((B, H, W, cin), dtype=torch.float32, device=dev())
    if cout < 32:
        zb = torch.zeros(cin, dtype=torch.float32, device=dev())
        _native.check(lib.pty_ws_conv3x3_direct(B, H, W, cout, cin, p(dz), p(wf), p(zb), 0, None, None, p(dx),
                                                stream()))
    else:
        _native.check(lib.pty_ws_conv3x3_tc_f32(B, H, W, cout, cin, p(dz), p(wf), p(dx), stream()))
    assert status_ok()
    ref = dgrad_ref(dz.float().cpu().numpy().astype(np.float64), wd.float().cpu().numpy().astype(np.float64))
    got = dx.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5


def shift_ref(x, S):
    """XS[s][c][p] of pty_ws_shift_transpose for NHWC x (float64)."""
    B, H, W, C = x.shape
    out = np.zeros((S, C, B, H, W))
    for s in range(S):
        sh = s - 1 if S == 3 else 0
        src = np.zeros_like(x)
        if sh < 0:
            src[:, :, 1:] = x[:, :, :-1]
        elif sh > 0:
            src[:, :, :-1] = x[:, :, 1:]
        else:
            src = x
        out[s] = np.transpose(src, (3, 0, 1, 2))
    return out.reshape(S, C, B * H * W)


@pytest.mark.parametrize("S,C", [(3, 64), (1, 2), (3, 32), (1, 128), (3, 128)])
@pytest.mark.parametrize("B,H,W", [(2, 8, 32), (1, 3, 34)])
def test_shift_transpose_matches_numpy(S, C, B, H, W):
    """Exact (a copy): whole 128-pixel tiles, and a ragged last tile with
    rows that straddle tiles (34 x 3 pixels)."""
    rng = np.random.default_rng(S * 100 + C)
    x = bf16(rng.standard_normal((B, H, W, C)))
    xs = torch.empty((S, C, B * H * W), dtype=torch.bfloat16, device=dev())
    _native.check(_native.load().pty_ws_shift_transpose(B, H, W, C, S, p(x), p(xs), stream()))
    ref = shift_ref(x.float().cpu().numpy().astype(np.float64), S)
    np.testing.assert_array_equal(xs.float().cpu().numpy(), ref)


def wgrad_ref(x, dz):
    """float64 dW[co][(ky*3+kx) C_in + ci] = sum_p dZ[p][co] X[p + (ky-1, kx-1)][ci]."""
    B, H, W, cin = x.shape
    co = dz.shape[-1]
    xp = np.zeros((B, H + 2, W + 2, cin))
    xp[:, 1:-1, 1:-1] = x
    dw = np.zeros((co, 3, 3, cin))
    for ky in range(3):
        for kx in range(3):
            dw[:, ky, kx] = np.einsum("bhwo,bhwc->oc", dz, xp[:, ky:ky + H, kx:kx + W])
    return dw.reshape(co, 9 * cin)


# (B, H, W, C_in, C_out): the network's layers 1-5 at 128^2 frames, plus a
# 192-wide image (three chunks per row) with C_out 48 (N = 48: a partial
# 32-column accumulator read)
WGRAD_CASES = [(2, 64, 64, 32, 64), (2, 32, 32, 64, 128), (2, 64, 64, 128, 64), (2, 128, 128, 64, 32),
               (2, 128, 128, 32, 2), (1, 16, 192, 64, 48)]


@pytest.mark.parametrize("case", WGRAD_CASES, ids=lambda c: "x".join(map(str, c)))
def test_wgrad_tc_matches_fp64(case):
    """pty_ws_wgrad_tc (tcgen05, pixels on K, split partial sums added in
    order) against the float64 weight gradient of the same BF16 operands:
    the products are exact in FP32, the sums run over up to 2^15 pixels per
    split, so within 1e-5 norm-wise; and the same bits on a second call."""
    B, H, W, cin, cout = case
    lib = _native.load()
    rng = np.random.default_rng(B + H + W + cin + cout)
    x = bf16(rng.standard_normal((B, H, W, cin)))
    dz = bf16(rng.standard_normal((B, H, W, cout)))
    P = B * H * W
    xs = torch.empty((3, cin, P), dtype=torch.bfloat16, device=dev())
    dzt = torch.empty((cout, P), dtype=torch.bfloat16, device=dev())
    _native.check(lib.pty_ws_shift_transpose(B, H, W, cin, 3, p(x), p(xs), stream()))
    _native.check(lib.pty_ws_shift_transpose(B, H, W, cout, 1, p(dz), p(dzt), stream()))
    n = int(lib.pty_ws_wgrad_tc_scratch(B, H, W, cin, cout))
    assert n > 0
    scr = torch.empty(n, dtype=torch.float32, device=dev())
    dws = []
    for _ in range(2):
        dw = torch.full((cout, 9 * cin), float("nan"), dtype=torch.float32, device=dev())
        _native.check(lib.pty_ws_wgrad_tc(B, H, W, cin, cout, p(xs), p(dzt), p(dw), p(scr), n, stream()))
        dws.append(dw.cpu().numpy())
    assert status_ok()
    ref = wgrad_ref(x.float().cpu().numpy().astype(np.float64), dz.float().cpu().numpy().astype(np.float64))
    got = dws[0].astype(np.float64)
    assert np.all(np.isfinite(got))
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5
    np.testing.assert_array_equal(dws[0], dws[1])


def test_wgrad_tc_rejects_unsupported_shapes():
    lib = _native.load()
    for args in ((1, 8, 64, 2, 32), (1, 8, 64, 48, 32), (1, 8, 16, 32, 32), (1, 8, 96, 32, 32),
                 (1, 8, 64, 32, 256)):
        assert lib.pty_ws_wgrad_tc_scratch(*args) == -1, args
    t = torch.zeros(1 << 16, dtype=torch.float32, device=dev())
    rc = lib.pty_ws_wgrad_tc(1, 8, 16, 32, 32, p(t), p(t), p(t), p(t), 1 << 16, stream())
    assert rc == 6


def _align_case(seed, side=5, M=32, step=16):
    rng = np.random.default_rng(seed)
    R = -np.array([(step * i, step * j) for i in range(side) for j in range(side)], dtype=np.int64)
    U = V = M + step * (side - 1)
    O = (0.6 + 0.4 * rng.random((U, V))) * np.exp(1j * rng.uniform(-1, 1, (U, V)))
    y, x = np.mgrid[:M, :M] - M // 2
    P = np.exp(-(x ** 2 + y ** 2) / (2 * 8.0 ** 2)) * np.exp(1j * 0.01 * (x ** 2 + y ** 2))
    return rng, R, O, P, U, V


def test_align_phase_matches_numpy():
    """pty_ws_align_phase against NumPy: z_f = sum psi_f conj(P O[window f]),
    psi_f * conj(z_f) / |z_f|; a frame whose window leaves the object is
    left unchanged."""
    rng, R, O, P, U, V = _align_case(1)
    n, M = len(R), P.shape[0]
    psi = rng.standard_normal((n, M, M)) + 1j * rng.standard_normal((n, M, M))
    win = (-R).astype(np.int32)
    win[3] = (U - M + 1, 0)                     # outside: unchanged
    want = psi.copy()
    for f in range(n):
        if f == 3:
            continue
        a, b = win[f]
        z = np.sum(psi[f] * np.conj(P * O[a:a + M, b:b + M]))
        want[f] = psi[f] * np.conj(z) / abs(z)
    # device copies held by name until the kernel has run
    psi_d = torch.from_numpy(psi.astype(np.complex64)).to(dev())
    win_d = torch.from_numpy(win).to(dev())
    O_d = torch.from_numpy(O.astype(np.complex64)).to(dev())
    P_d = torch.from_numpy(P.astype(np.complex64)).to(dev())
    lib = _native.load()
    _native.check(lib.pty_ws_align_phase(n, M, M, p(win_d), U, V, p(O_d), p(P_d), p(psi_d), stream()))
    got = psi_d.cpu().numpy().astype(np.complex128)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-5
    np.testing.assert_array_equal(got[3], psi[3].astype(np.complex64))


def test_align_phase_removes_frame_offsets():
    """Exact exit waves of a known object under random per-frame phase
    offsets of up to 0.5 rad (what a network that cannot see a frame's
    constant phase produces): stitch, then align and stitch again.  The
    alternation is a power iteration over the frames' overlap graph, so it
    removes the offsets gradually: NumPy runs of the same steps on this case
    give object errors (after one global phase) 0.243, 0.140 after two
    alignments and 0.036 after twenty."""
    from gpu_util import Plan
    rng, R, O, P, U, V = _align_case(2)
    n, M = len(R), P.shape[0]
    theta = rng.uniform(-0.5, 0.5, n)
    psi = np.stack([P * O[-r0:-r0 + M, -r1:-r1 + M] * np.exp(1j * t) for (r0, r1), t in zip(R, theta)])
    plan = Plan(n, M, M, U, V, R)
    try:
        lib = _native.load()
        psi_d = torch.from_numpy(psi.astype(np.complex64)).to(dev())
        P_d = torch.from_numpy(P.astype(np.complex64)).to(dev())
        O_d = torch.empty((U, V), dtype=torch.complex64, device=dev())
        heat = torch.empty((U, V), dtype=torch.float64, device=dev())
        win = torch.from_numpy((-R).astype(np.int32)).to(dev())

        def err():
            o = O_d.cpu().numpy().astype(np.complex128)
            c = np.vdot(o, O)                   # best global phase
            return np.linalg.norm(o * c / abs(c) - O) / np.linalg.norm(O)
        _native.check(lib.pty_psup_O(plan.h, p(psi_d), p(P_d), p(heat), 1, 1e-10, p(O_d), stream()))
        es = [err()]
        for _ in range(20):
            _native.check(lib.pty_ws_align_phase(n, M, M, p(win), U, V, p(O_d), p(P_d), p(psi_d), stream()))
            _native.check(lib.pty_psup_O(plan.h, p(psi_d), p(P_d), p(heat), 0, 1e-10, p(O_d), stream()))
            es.append(err())
    finally:
        plan.close()
    assert abs(es[0] - 0.243) < 0.01 and abs(es[2] - 0.140) < 0.01 and abs(es[20] - 0.036) < 0.005, es


def test_conv_tc_rejects_unsupported_shapes():
    lib = _native.load()
    t = torch.zeros(1 << 16, dtype=torch.bfloat16, device=dev())
    bd = torch.zeros(256, dtype=torch.float32, device=dev())
    for args in ((1, 8, 8, 48, 32), (1, 8, 8, 64, 48), (1, 8, 8, 64, 256), (1, 8, 96, 64, 32)):
        rc = lib.pty_ws_conv3x3_tc(*args, p(t), p(t), p(bd), 1, None, p(t), None, stream())
        assert rc == 6, args


def test_inference_pass_matches_im2col_network():
    """The network's inference pass with layers 1-4 on the tensor cores gives
    the im2col path's outputs (128^2 frames, random network and inputs)."""
    net = WarmStartNet(128, 128, seed=3, device=dev())
    rng = np.random.default_rng(5)
    x = bf16(rng.standard_normal((4, 128, 128, 2)))
    y_old = net.forward(x).clone()
    y_tc = net.forward_infer(x).clone()
    torch.cuda.synchronize()
    assert status_ok()
    a, b = y_tc.cpu().numpy(), y_old.cpu().numpy()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-2
    assert len(LAYERS) == 6


@pytest.mark.parametrize("case", [(2, 128, 128, 2, 32, True), (2, 128, 128, 32, 2, False),
                                  (1, 16, 24, 8, 16, True), (1, 9, 15, 4, 8, True), (1, 6, 10, 32, 2, False)],
                         ids=lambda c: "x".join(map(str, c[:5])))
def test_conv_direct_matches_fp64(case):
    """The CUDA-core direct convolution (the network's 2-channel layers) against
    the float64 reference of the same BF16 operands, for both its outputs: the
    FP32 pre-rounding values (out32) and the BF16 activation with a skip."""
    B, H, W, cin, cout, relu = case
    lib = _native.load()
    rng = np.random.default_rng(H + cin + cout)
    x = rng.standard_normal((B, H, W, cin)).astype(np.float32)
    w = (rng.standard_normal((cout, 9 * cin)) * np.sqrt(2.0 / (9 * cin))).astype(np.float32)
    b = (0.1 * rng.standard_normal(cout)).astype(np.float32)
    sk = rng.standard_normal((B, H, W, cout)).astype(np.float32)
    xd, wd, skd = bf16(x), bf16(w), bf16(sk)
    bd = torch.from_numpy(b).to(dev())
    out = torch.empty((B, H, W, cout), dtype=torch.bfloat16, device=dev())
    out32 = torch.empty((B, H, W, cout), dtype=torch.float32, device=dev())
    _native.check(lib.pty_ws_conv3x3_direct(B, H, W, cin, cout, p(xd), p(wd), p(bd), int(relu), p(skd),
                                            p(out), p(out32), stream()))
    xr = xd.float().cpu().numpy().astype(np.float64)
    wr = wd.float().cpu().numpy().astype(np.float64)
    skr = skd.float().cpu().numpy().astype(np.float64)
    # FP32 output: sums of exact BF16 products, FP32 accumulation (~1e-6)
    B_, H_, W_ = B, H, W
    xp = np.zeros((B_, H_ + 2, W_ + 2, cin))
    xp[:, 1:-1, 1:-1] = xr
    z = np.zeros((B_, H_, W_, cout))
    wk = wr.reshape(cout, 3, 3, cin)
    for ky in range(3):
        for kx in range(3):
            z += np.einsum("bhwc,oc->bhwo", xp[:, ky:ky + H_, kx:kx + W_], wk[:, ky, kx])
    z += b
    if relu:
        z = np.maximum(z, 0)
    got32 = out32.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(got32 - z) / np.linalg.norm(z) < 1e-5
    ref = conv_ref(xr, wr, b.astype(np.float64), relu, skr)
    got = out.float().cpu().numpy().astype(np.float64)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 3e-3


@pytest.mark.parametrize("case", [(2, 128, 128, False), (1, 5, 64, True), (1, 6, 40, False)],
                         ids=lambda c: "x".join(map(str, c[:3])))
def test_conv_direct_last_layer_matches_fp64(case):
    """The network's last layer (32 -> 2 channels, FP32 output only): the
    four-lanes-per-pixel kernel with packed FP32x2 FMAs when W is a multiple
    of 32 (the 40-wide case takes the general kernel), against float64 of the
    same BF16 operands: FP32 accumulation in another order, within 1e-5."""
    B, H, W, relu = case
    cin, cout = 32, 2
    lib = _native.load()
    rng = np.random.default_rng(H + W)
    xd = bf16(rng.standard_normal((B, H, W, cin)))
    wd = bf16(rng.standard_normal((cout, 9 * cin)) * np.sqrt(2.0 / (9 * cin)))
    b = (0.1 * rng.standard_normal(cout)).astype(np.float32)
    bd = torch.from_numpy(b).to(dev())
    out32 = torch.full((B, H, W, cout), float("nan"), dtype=torch.float32, device=dev())
    _native.check(lib.pty_ws_conv3x3_direct(B, H, W, cin, cout, p(xd), p(wd), p(bd), int(relu), None, None,
                                            p(out32), stream()))
    xr = xd.float().cpu().numpy().astype(np.float64)
    wr = wd.float().cpu().numpy().astype(np.float64)
    xp = np.zeros((B, H + 2, W + 2, cin))
    xp[:, 1:-1, 1:-1] = xr
    z = np.zeros((B, H, W, cout))
    wk = wr.reshape(cout, 3, 3, cin)
    for ky in range(3):
        for kx in range(3):
            z += np.einsum("bhwc,oc->bhwo", xp[:, ky:ky + H, kx:kx + W], wk[:, ky, kx])
    z += b
    if relu:
        z = np.maximum(z, 0)
    got = out32.cpu().numpy().astype(np.float64)
    assert np.all(np.isfinite(got))
    assert np.linalg.norm(got - z) / np.linalg.norm(z) < 1e-5


def test_conv_direct_rejects_unsupported_shapes():
    lib = _native.load()
    t = torch.zeros(1 << 16, dtype=torch.bfloat16, device=dev())
    bd = torch.zeros(64, dtype=torch.float32, device=dev())
    for cin, cout in ((3, 8), (64, 8), (2, 64), (2, 3)):
        rc = lib.pty_ws_conv3x3_direct(1, 8, 8, cin, cout, p(t), p(t), p(bd), 1, None, p(t), None, stream())
        assert rc != 0, (cin, cout)


def test_crop_and_upsample_match_numpy():
    lib = _native.load()
    rng = np.random.default_rng(8)
    I = rng.random((3, 32, 32)).astype(np.float32)
    Id = torch.from_numpy(I).to(dev())
    out = torch.empty((3, 16, 16), dtype=torch.float32, device=dev())
    _native.check(lib.pty_ws_crop_center(3, 32, 32, 16, 16, p(Id), None, 0.5, p(out), None, stream()))
    np.testing.assert_array_equal(out.cpu().numpy(), 0.5 * I[:, 8:24, 8:24])
    sel = torch.tensor([2, 0], dtype=torch.int32, device=dev())
    out2 = torch.empty((2, 16, 16), dtype=torch.float32, device=dev())
    _native.check(lib.pty_ws_crop_center(2, 32, 32, 16, 16, p(Id), p(sel), 1.0, p(out2), stream()))
    np.testing.assert_array_equal(out2.cpu().numpy(), I[[2, 0], 8:24, 8:24])
    Oh = (rng.standard_normal((7, 9)) + 1j * rng.standard_normal((7, 9))).astype(np.complex64)
    Ohd = torch.from_numpy(Oh).to(dev())
    U, V, f = 15, 20, 2
    O = torch.empty((U, V), dtype=torch.complex64, device=dev())
    _native.check(lib.pty_ws_upsample_object(7, 9, p(Ohd), U, V, f, p(O), stream()))
    su = np.minimum(np.arange(U) / f, 6.0)
    sv = np.minimum(np.arange(V) / f, 8.0)
    u0, v0 = np.floor(su).astype(int), np.floor(sv).astype(int)
    u1, v1 = np.minimum(u0 + 1, 6), np.minimum(v0 + 1, 8)
    du, dv = (su - u0)[:, None], (sv - v0)[None, :]
    ref = ((1 - du) * (1 - dv) * Oh[u0][:, v0] + (1 - du) * dv * Oh[u0][:, v1]
           + du * (1 - dv) * Oh[u1][:, v0] + du * dv * Oh[u1][:, v1])
    np.testing.assert_allclose(O.cpu().numpy(), ref, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("cover,graph", [(True, True), (False, False)])
def test_downsampled_start_sees_the_object(cover, graph):
    """The warm start for 256^2 frames through a 128^2 network (untrained, so
    only the geometry is checked): the stitched, upsampled object has the full
    grid's shape and is finite; where frames overlap it is non-zero, and
    everywhere it is a weighted mean of the network's unit phasors (weights
    |P|^2 of the resampled probe), so its modulus is at most 1."""
    from ptychography_gb300 import warmstart as ws
    net = WarmStartNet(128, 128, seed=1, device=dev())
    rng = np.random.default_rng(3)
    N, U = 256, 384
    O_true = ws.random_object(rng, U)
    P = ws.aperture_probe(N, 60, 8, 0.0005)
    R = -np.array([(i, j) for i in range(0, 129, 32) for j in range(0, 129, 32)], dtype=np.int64)
    from gpu_util import Plan
    plan = Plan(len(R), N, N, U, U, R)
    Od = torch.from_numpy(O_true.astype(np.complex64)).to(dev())
    Pd = torch.from_numpy(P.astype(np.complex64)).to(dev())
    I = torch.empty((len(R), N, N), dtype=torch.float32, device=dev())
    _native.check(_native.load().pty_intensities(plan.h, p(Od), p(Pd), p(I), stream()))
    st = ws.DownsampledStart(net, len(R), N, N, P, R, cover=cover, graph=graph)
    assert (len(st.frames) < len(R)) == cover
    O = st.run(I, U, U)
    o = O.cpu().numpy()
    o2 = st.run(I, U, U).cpu().numpy()          # a graph replay gives the same object
    st.close()
    plan.close()
    np.testing.assert_array_equal(o, o2)
    assert o.shape == (U, U) and np.all(np.isfinite(o))
    assert np.abs(o[128:256, 128:256]).min() > 0
    assert np.abs(o).max() <= 1.0 + 1e-4


def test_training_forward_on_tensor_cores_gives_the_same_gradients():
    """A training step whose forward pass runs on the tensor cores
    (forward_train: layers 1-4 on pty_ws_conv3x3_tc keeping their
    activations, the backward pass forming its own im2col buffers) gives the
    weight and bias gradients of the im2col + mma.sync forward pass, up to
    the FP32 summation order of the forward sums (one BF16 rounding step on
    some activations) and of the input and weight gradients (flipped-weight
    convolutions instead of GEMM + col2im; the tensor-core weight gradient
    for layers 1-5): within 3e-2 norm-wise per layer."""
    net = WarmStartNet(128, 128, seed=4, device=dev())
    rng = np.random.default_rng(9)
    B = 8
    x = bf16(rng.standard_normal((B, 128, 128, 2)) * 0.5)
    t = torch.from_numpy(rng.standard_normal((B, 128, 128, 2)).astype(np.float32)).to(dev())
    wgt = torch.full((B, 128, 128), 1.0 / (B * 128 * 128), dtype=torch.float32, device=dev())
    grads = []
    for train in (False, True):
        y = net.forward_train(x) if train else net.forward(x)
        parts, dy = net.loss_grad(y, t, wgt)
        net.backward(dy)
        torch.cuda.synchronize()
        grads.append(([g.clone() for g in net.gw], [g.clone() for g in net.gb], float(parts.sum().cpu())))
    assert status_ok()
    (gw0, gb0, l0), (gw1, gb1, l1) = grads
    assert abs(l1 - l0) < 1e-2 * abs(l0)
    for i in range(len(LAYERS)):
        ew = float((gw1[i] - gw0[i]).norm() / gw0[i].norm())
        eb = float((gb1[i] - gb0[i]).norm() / (gb0[i].norm() + 1e-30))
        assert ew < 3e-2 and eb < 3e-2, (i, ew, eb)
