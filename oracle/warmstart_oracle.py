"""CPU oracle for the learned warm start's network.

TEST INFRASTRUCTURE ONLY.  The GPU tests call it to produce the expected
forward pass, gradients, loss, Adam step and data preparation of the network
that ``ptychography_gb300.warmstart`` runs on the library's ``pty_ws_*``
kernels; the shipped engine never imports it.

The warm start has no counterpart in the reference (whose ERA starts from an
object of ones, era.py:480-486), so nothing of the reference's can pin this
restatement.  It is instead pinned on the CPU against torch's float64
autograd of the same network (``tests/test_warmstart_oracle_cpu.py``), and the
device's passes are checked against it (``tests/test_gpu_warmstart.py``).

The network (activations NHWC, weights [C_out][3][3][C_in] flattened to
[C_out][9 C_in], "same" zero padding, cross-correlation as in torch; the
input x has two channels, the real and imaginary parts of the frame's
back-projected object estimate, ``bp_input``):

    h1 = relu(conv0(x))
    h2 = relu(conv1(pool(h1)))
    h3 = relu(conv2(pool(h2)))
    h4 = relu(conv3(up(h3))) + h2
    h5 = relu(conv4(up(h4))) + h1
    y  = conv5(h5)

With ``bf16=True`` every value the device stores as BF16 is rounded to BF16
(round to nearest, ties to even) at the same point: the input, the weights,
each activation, each pooled and skip-summed map, and the activation gradients
that feed the weight- and input-gradient products.  What then remains between
the device and the oracle is the order of the FP32 accumulations.
"""
import numpy as np

__all__ = ["LAYERS", "bf16_round", "im2col", "col2im", "pool2", "pool2_bwd", "up2", "up2_bwd",
           "init_weights", "forward", "backward", "loss_grad", "adam", "bp_input", "targets", "exits"]

# (C_in, C_out, relu, level) of the six convolutions (level = log2 of the
# downsampling at which the layer runs)
LAYERS = ((2, 32, True, 0), (32, 64, True, 1), (64, 128, True, 2),
          (128, 64, True, 1), (64, 32, True, 0), (32, 2, False, 0))


def bf16_round(x):
    """Round to BF16 (the top 16 bits of an IEEE single), nearest, ties to even,
    returned as float64.  The value is first rounded to single precision, as
    the device holds it before its own conversion."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _identity(x):
    return np.asarray(x, dtype=np.float64)


def im2col(x):
    """(B, H, W, C) -> (B H W, 9 C); column (ky 3 + kx) C + c holds
    x[b, y + ky - 1, x + kx - 1, c], zero outside the frame."""
    B, H, W, C = x.shape
    xp = np.zeros((B, H + 2, W + 2, C), dtype=np.float64)
    xp[:, 1:H + 1, 1:W + 1] = x
    cols = [xp[:, ky:ky + H, kx:kx + W, :] for ky in range(3) for kx in range(3)]
    return np.concatenate(cols, axis=-1).reshape(B * H * W, 9 * C)


def col2im(dcol, B, H, W, C):
    """Adjoint of im2col: (B H W, 9 C) -> (B, H, W, C)."""
    d = np.asarray(dcol, dtype=np.float64).reshape(B, H, W, 9, C)
    xp = np.zeros((B, H + 2, W + 2, C), dtype=np.float64)
    for ky in range(3):
        for kx in range(3):
            xp[:, ky:ky + H, kx:kx + W, :] += d[:, :, :, 3 * ky + kx, :]
    return xp[:, 1:H + 1, 1:W + 1]


def pool2(x):
    """2 x 2 average pooling, (B, H, W, C) -> (B, H/2, W/2, C)."""
    return 0.25 * (x[:, 0::2, 0::2] + x[:, 0::2, 1::2] + x[:, 1::2, 0::2] + x[:, 1::2, 1::2])


def pool2_bwd(dy):
    """Adjoint of pool2: each input pixel receives a quarter of its output's gradient."""
    return 0.25 * np.repeat(np.repeat(dy, 2, axis=1), 2, axis=2)


def up2(x):
    """Nearest 2 x upsampling, (B, h, w, C) -> (B, 2h, 2w, C)."""
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up2_bwd(dy):
    """Adjoint of up2: the sum of each 2 x 2 block."""
    return dy[:, 0::2, 0::2] + dy[:, 0::2, 1::2] + dy[:, 1::2, 0::2] + dy[:, 1::2, 1::2]


def init_weights(seed=0):
    """He-initialised weights ([C_out][9 C_in], float32) and zero biases, drawn
    as the library's network draws them (numpy default_rng(seed), one
    standard-normal block per layer in layer order)."""
    rng = np.random.default_rng(seed)
    w, b = [], []
    for cin, cout, _, _ in LAYERS:
        std = float(np.sqrt(2.0 / (9 * cin)))
        w.append((rng.standard_normal((cout, 9 * cin)) * std).astype(np.float32))
        b.append(np.zeros(cout, dtype=np.float32))
    return w, b


def _conv(i, x, w, b, q, skip=None, last=False):
    """One layer: returns (out, cache) with out = act(conv(x) + bias) (+ skip)."""
    cin, cout, relu, _ = LAYERS[i]
    B, H, W, _ = x.shape
    col = im2col(x)
    wq = q(w[i])
    z = col @ wq.T + np.asarray(b[i], dtype=np.float64)
    if last:
        return z.reshape(B, H, W, cout), {"col": col, "wq": wq, "a": None, "shape": (B, H, W)}
    if relu:
        z = np.maximum(z, 0.0)
    a = q(z).reshape(B, H, W, cout)
    out = a if skip is None else q(a + skip)
    return out, {"col": col, "wq": wq, "a": a, "shape": (B, H, W)}


def forward(x, w, b, bf16=False):
    """x: (B, H, W, 2) network input; w, b: the six layers' weights and biases.
    Returns y (B, H, W, 2) and the cache the backward pass needs."""
    q = bf16_round if bf16 else _identity
    x = q(x)
    cache = []
    h1, c = _conv(0, x, w, b, q)
    cache.append(c)
    h2, c = _conv(1, q(pool2(h1)), w, b, q)
    cache.append(c)
    h3, c = _conv(2, q(pool2(h2)), w, b, q)
    cache.append(c)
    h4, c = _conv(3, up2(h3), w, b, q, skip=h2)
    cache.append(c)
    h5, c = _conv(4, up2(h4), w, b, q, skip=h1)
    cache.append(c)
    y, c = _conv(5, h5, w, b, q, last=True)
    cache.append(c)
    return y, {"layers": cache, "bf16": bf16}


def _conv_bwd(i, c, dA, q, need_dx):
    cin, cout, relu, _ = LAYERS[i]
    B, H, W = c["shape"]
    g = np.asarray(dA, dtype=np.float64).reshape(B * H * W, cout)
    if relu:
        g = g * (c["a"].reshape(B * H * W, cout) > 0)
    gb = g.sum(axis=0)
    gq = q(g)
    gw = gq.T @ c["col"]
    dx = col2im(gq @ c["wq"], B, H, W, cin) if need_dx else None
    return gw, gb, dx


def backward(cache, dy):
    """Gradients of the six layers' weights and biases (lists in layer order)
    for the output gradient dy (B, H, W, 2), and the input gradient."""
    q = bf16_round if cache["bf16"] else _identity
    L = cache["layers"]
    gw, gb = [None] * 6, [None] * 6
    gw[5], gb[5], dh5 = _conv_bwd(5, L[5], dy, q, True)          # h5 = a4 + h1
    gw[4], gb[4], du4 = _conv_bwd(4, L[4], dh5, q, True)
    dh4 = up2_bwd(du4)                                           # h4 = a3 + h2
    gw[3], gb[3], du3 = _conv_bwd(3, L[3], dh4, q, True)
    gw[2], gb[2], dp2 = _conv_bwd(2, L[2], up2_bwd(du3), q, True)
    dh2 = pool2_bwd(dp2) + dh4
    gw[1], gb[1], dp1 = _conv_bwd(1, L[1], dh2, q, True)
    dh1 = pool2_bwd(dp1) + dh5
    gw[0], gb[0], dx = _conv_bwd(0, L[0], dh1, q, True)
    return gw, gb, dx


def loss_grad(y, t, weight):
    """Weighted squared error sum_p weight[p] |y[p] - t[p]|^2 over the (cos, sin)
    pairs, and its gradient 2 weight (y - t)."""
    e = np.asarray(y, np.float64) - np.asarray(t, np.float64)
    wgt = np.asarray(weight, np.float64)[..., None]
    return float(np.sum(wgt * e * e)), 2.0 * wgt * e


def adam(w, g, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma and Ba, 2015, Algorithm 1) with bias correction;
    returns the new (w, m, v)."""
    w, g, m, v = (np.asarray(a, np.float64) for a in (w, g, m, v))
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return w - lr * mh / (np.sqrt(vh) + eps), m, v


def bp_input(I, P):
    """Network input for centred intensities I (n, H, W) under the probe P
    (H, W): the back-projection bp = ifftn(sqrt(I) exp(i angle(fftn P))) with
    the amplitudes in natural FFT order (Back_projection's exit waves,
    back_projection.py:74-78), then z = bp conj(P) / (max|P|^2 r) with
    r = sqrt(sum |bp|^2 / sum |P|^2) per frame (1 for an empty frame);
    returns (n, H, W, 2) = (Re z, Im z)."""
    amp = np.fft.ifftshift(np.sqrt(np.maximum(np.asarray(I, np.float64), 0.0)), axes=(-2, -1))
    P = np.asarray(P, np.complex128)
    bp = np.fft.ifftn(amp * np.exp(1j * np.angle(np.fft.fftn(P))), axes=(-2, -1))
    sb = np.sum(np.abs(bp) ** 2, axis=(-2, -1))
    sp = np.sum(np.abs(P) ** 2)
    r = np.where(sb > 0, np.sqrt(sb / sp), 1.0)
    z = bp * np.conj(P) / (np.max(np.abs(P) ** 2) * r[:, None, None])
    return np.stack([z.real, z.imag], axis=-1)


def targets(psi, P, object_phase=True, wscale=1.0):
    """Training targets for exit waves psi (n, H, W) under the probe P (H, W):
    (cos, sin) of arg psi, or of arg psi conj(P) (the object's phase under the
    probe) when object_phase; (1, 0) where the wave is 0.  Weights |P|^2 wscale."""
    v = np.asarray(psi, np.complex128)
    if object_phase:
        v = v * np.conj(np.asarray(P, np.complex128))
    r = np.abs(v)
    nz = r > 0
    c = np.where(nz, v.real / np.where(nz, r, 1.0), 1.0)
    s = np.where(nz, v.imag / np.where(nz, r, 1.0), 0.0)
    wgt = np.broadcast_to(np.abs(np.asarray(P, np.complex128)) ** 2 * wscale, v.shape)
    return np.stack([c, s], axis=-1), np.array(wgt)


def exits(y, P, object_phase=True):
    """Exit waves with the predicted phases y (n, H, W, 2) = (cos, sin), up to
    scale: P e^{i phase} when object_phase, else |P| e^{i phase}; a zero
    prediction reads as phase 0."""
    y = np.asarray(y, np.float64)
    r = np.hypot(y[..., 0], y[..., 1])
    nz = r > 0
    ph = np.where(nz, y[..., 0] / np.where(nz, r, 1.0), 1.0) + 1j * np.where(nz, y[..., 1] / np.where(nz, r, 1.0), 0.0)
    P = np.asarray(P, np.complex128)
    return (P if object_phase else np.abs(P)) * ph
