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
# plus a 256-wide image (two tiles per row) and a 32-channel-in layer with skip
CASES = [(2, 64, 64, 32, 64, True, False), (2, 32, 32, 64, 128, True, False),
         (2, 64, 64, 128, 64, True, True), (2, 128, 128, 64, 32, True, True),
         (1, 8, 256, 64, 96, False, False), (3, 16, 16, 32, 32, True, True)]


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
                                        p(out), stream()))
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


def test_conv_tc_rejects_unsupported_shapes():
    lib = _native.load()
    t = torch.zeros(1 << 16, dtype=torch.bfloat16, device=dev())
    bd = torch.zeros(256, dtype=torch.float32, device=dev())
    for args in ((1, 8, 8, 48, 32), (1, 8, 8, 64, 48), (1, 8, 8, 64, 256), (1, 8, 96, 64, 32)):
        rc = lib.pty_ws_conv3x3_tc(*args, p(t), p(t), p(bd), 1, None, p(t), stream())
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
