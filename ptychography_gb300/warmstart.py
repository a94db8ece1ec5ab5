"""Learned warm start: a small conv encoder-decoder predicts each frame's
object phase under the probe from the frame's back-projection; the predicted
exit waves are stitched into an initial object (the overlap update,
era.py:336-369) from which ERA starts instead of from ones (era.py:480-486).
No reference counterpart.

The input is local in the object: the back-projection
bp = ifftn(sqrt(I) exp(i angle(fftn P))) (Back_projection's exit waves,
back_projection.py:74-78, with the amplitudes in natural FFT order) gives
bp conj(P) ~ |P|^2 (1 + i phase / 2 + a defocused twin term) for a weak phase
object under a probe with a quadratic phase, so 3 x 3 convolutions with a
receptive field of a few tens of pixels can refine it.  sqrt(I) itself would
need the whole pattern for every output pixel.

The network (6 layers, 3 x 3 kernels, 32-128 channels, BF16 weights and
activations, FP32 accumulation) runs forward and backward on the library's
kernels (``pty_ws_*``: im2col + BF16 tensor-core GEMMs, pooling, upsampling,
activations, loss, Adam); torch only holds device memory.

    x  = bp conj(P) / (max|P|^2 r), r the RMS amplitude     H x W x 2  (Re, Im)
    h1 = relu(conv(x))                                    H x W x 32
    h2 = relu(conv(pool(h1)))                             H/2 x W/2 x 64
    h3 = relu(conv(pool(h2)))                             H/4 x W/4 x 128
    h4 = relu(conv(up(h3))) + h2                          H/2 x W/2 x 64
    h5 = relu(conv(up(h4))) + h1                          H x W x 32
    y  = conv(h5)                                         H x W x 2  (cos, sin of the phase)
"""
import ctypes

import numpy as np

from . import _native

# (C_in, C_out, relu, level) of the six convolutions; level = log2 of the
# downsampling
LAYERS = ((2, 32, True, 0), (32, 64, True, 1), (64, 128, True, 2),
          (128, 64, True, 1), (64, 32, True, 0), (32, 2, False, 0))


def _torch():
    import torch
    return torch


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class WarmStartNet:
    """Parameters (FP32 masters, BF16 copies, Adam moments) and the
    forward / backward passes for frames of H x W pixels (H, W multiples of 4)."""

    def __init__(self, H, W, seed=0, device=None, object_phase=True):
        torch = _torch()
        # target: the object's phase under the probe (the exit-wave phase less
        # the probe's, which a known probe restores at stitching), or the
        # exit-wave phase itself
        self.object_phase = bool(object_phase)
        if H % 4 or W % 4:
            raise ValueError("frame sides must be multiples of 4")
        self.H, self.W = H, W
        self.dev = device or torch.device("cuda", torch.cuda.current_device())
        self.lib = _native.load()
        rng = np.random.default_rng(seed)
        self.w, self.b, self.wb = [], [], []
        for cin, cout, _, _ in LAYERS:
            std = float(np.sqrt(2.0 / (9 * cin)))                 # He initialisation
            w = (rng.standard_normal((cout, 9 * cin)) * std).astype(np.float32)
            self.w.append(torch.from_numpy(w).to(self.dev))
            self.b.append(torch.zeros(cout, dtype=torch.float32, device=self.dev))
            self.wb.append(torch.empty((cout, 9 * cin), dtype=torch.bfloat16, device=self.dev))
        self.m = [torch.zeros_like(t) for t in self.w + self.b]
        self.v = [torch.zeros_like(t) for t in self.w + self.b]
        self.step_count = 0
        self._sync_bf16()
        self._bufs = {}
        self._zero_bias = torch.zeros(128, dtype=torch.float32, device=self.dev)

    def _sp(self):
        torch = _torch()
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def _sync_bf16(self):
        for w, wb in zip(self.w, self.wb):
            assert w.dtype == _torch().float32 and wb.dtype == _torch().bfloat16
            _native.check(self.lib.pty_ws_to_bf16(w.numel(), _p(w), _p(wb), self._sp()))

    def state_dict(self):
        return {"w": [t.cpu().numpy() for t in self.w], "b": [t.cpu().numpy() for t in self.b]}

    def load_state_dict(self, st):
        torch = _torch()
        for i in range(len(LAYERS)):
            self.w[i].copy_(torch.from_numpy(np.asarray(st["w"][i], np.float32)))
            self.b[i].copy_(torch.from_numpy(np.asarray(st["b"][i], np.float32)))
        self._sync_bf16()

    def _buf(self, name, shape, dtype):
        torch = _torch()
        t = self._bufs.get(name)
        n = int(np.prod(shape))
        if t is None or t.numel() < n or t.dtype != dtype:
            t = torch.empty(n, dtype=dtype, device=self.dev)
            self._bufs[name] = t
        return t[:n].view(*shape)

    # ------------------------------------------------------------ layers
    def _conv_fwd(self, i, x, B, H, W, skip=None, last=False):
        """x: (B, H, W, C_in) bf16 -> (a, out) bf16, or the FP32 output if last."""
        torch = _torch()
        cin, cout, relu, _ = LAYERS[i]
        lib, sp = self.lib, self._sp()
        P, K = B * H * W, 9 * cin
        col = self._buf("col%d" % i, (P, K), torch.bfloat16)
        _native.check(lib.pty_ws_im2col(B, H, W, cin, _p(x), _p(col), sp))
        Z = self._buf("z%d" % i, (P, cout), torch.float32)
        _native.check(lib.pty_ws_gemm(P, cout, K, _p(col), K, 1, _p(self.wb[i]), 1, K,
                                      _p(Z), cout, 1, 1, None, sp))
        if last:
            y = self._buf("y", (B, H, W, cout), torch.float32)
            _native.check(lib.pty_ws_bias_act(P, cout, _p(Z), _p(self.b[i]), 0, None, None, None,
                                              _p(y), sp))
            return y
        a = self._buf("a%d" % i, (B, H, W, cout), torch.bfloat16)
        out = self._buf("h%d" % i, (B, H, W, cout), torch.bfloat16) if skip is not None else a
        _native.check(lib.pty_ws_bias_act(P, cout, _p(Z), _p(self.b[i]), int(relu), _p(skip), _p(a),
                                          _p(out) if skip is not None else None, None, sp))
        return out

    def forward(self, x):
        """x: (B, H, W, 1) bf16 device tensor (normalised sqrt(I)); returns y
        (B, H, W, 2) float32, (cos, sin) of the predicted phase (unnormalised)."""
        torch = _torch()
        B, H, W = x.shape[0], self.H, self.W
        lib, sp = self.lib, self._sp()
        self._x = x
        self._fwd_inputs = None          # the im2col path keeps its own col buffers
        h1 = self._conv_fwd(0, x, B, H, W)
        p1 = self._buf("p1", (B, H // 2, W // 2, 32), torch.bfloat16)
        _native.check(lib.pty_ws_pool2(B, H, W, 32, _p(h1), _p(p1), sp))
        h2 = self._conv_fwd(1, p1, B, H // 2, W // 2)
        p2 = self._buf("p2", (B, H // 4, W // 4, 64), torch.bfloat16)
        _native.check(lib.pty_ws_pool2(B, H // 2, W // 2, 64, _p(h2), _p(p2), sp))
        h3 = self._conv_fwd(2, p2, B, H // 4, W // 4)
        u3 = self._buf("u3", (B, H // 2, W // 2, 128), torch.bfloat16)
        _native.check(lib.pty_ws_up2(B, H // 4, W // 4, 128, _p(h3), _p(u3), sp))
        h4 = self._conv_fwd(3, u3, B, H // 2, W // 2, skip=h2)
        u4 = self._buf("u4", (B, H, W, 64), torch.bfloat16)
        _native.check(lib.pty_ws_up2(B, H // 2, W // 2, 64, _p(h4), _p(u4), sp))
        h5 = self._conv_fwd(4, u4, B, H, W, skip=h1)
        return self._conv_fwd(5, h5, B, H, W, last=True)

    def _conv_tc(self, i, x, B, H, W, skip=None, keep=False):
        """Layer i on the tensor-core implicit-GEMM convolution (bias,
        activation and skip fused): x (B, H, W, C_in) bf16 -> (B, H, W, C_out) bf16.
        With keep (a training pass) the activation before the skip goes to the
        layer's "a%d" buffer for the backward pass."""
        torch = _torch()
        cin, cout, relu, _ = LAYERS[i]
        out = self._buf("t%d" % i, (B, H, W, cout), torch.bfloat16)
        act = None
        if keep:
            act = self._buf("a%d" % i, (B, H, W, cout), torch.bfloat16) if skip is not None else out
            if skip is None:
                self._bufs["a%d" % i] = out.view(-1)
        _native.check(self.lib.pty_ws_conv3x3_tc(B, H, W, cin, cout, _p(x), _p(self.wb[i]), _p(self.b[i]),
                                                 int(relu), _p(skip), _p(out),
                                                 _p(act) if skip is not None else None, self._sp()))
        return out

    def _tc_supported(self, B):
        """Whether layers 1-4 fit the tensor-core convolution's tile rules at
        this frame size (W at least 8 and dividing 128, H a multiple of
        128 / W, or W a multiple of 128)."""
        ok = True
        for H, W in ((self.H // 2, self.W // 2), (self.H // 4, self.W // 4), (self.H, self.W)):
            ok = ok and W >= 8 and ((W < 128 and 128 % W == 0 and H % (128 // W) == 0) or W % 128 == 0)
        return ok

    def forward_train(self, x):
        """The forward pass of a training step on the tensor cores: layers 1-4
        on pty_ws_conv3x3_tc (keeping each layer's activation for the
        backward pass), the 2-channel layers on the direct convolution;
        backward() then takes the weight gradients of layers 1-5 on the
        tensor cores too (pty_ws_wgrad_tc, from channel-major copies of the
        layer inputs; layer 0's 2-channel input through im2col + mma.sync)
        and the input gradients on the same convolutions (flipped weights,
        FP32 output).
        Falls back to forward() (im2col + mma.sync) where the frame size does
        not fit the tensor-core tiles.  x: (B, H, W, 2) bf16; returns y."""
        torch = _torch()
        B, H, W = x.shape[0], self.H, self.W
        if not self._tc_supported(B):
            self._fwd_inputs = None
            return self.forward(x)
        lib, sp = self.lib, self._sp()
        self._x = x
        h1 = self._conv_direct(0, x, B, H, W)
        self._bufs["a0"] = h1.view(-1)
        p1 = self._buf("p1", (B, H // 2, W // 2, 32), torch.bfloat16)
        _native.check(lib.pty_ws_pool2(B, H, W, 32, _p(h1), _p(p1), sp))
        h2 = self._conv_tc(1, p1, B, H // 2, W // 2, keep=True)
        p2 = self._buf("p2", (B, H // 4, W // 4, 64), torch.bfloat16)
        _native.check(lib.pty_ws_pool2(B, H // 2, W // 2, 64, _p(h2), _p(p2), sp))
        h3 = self._conv_tc(2, p2, B, H // 4, W // 4, keep=True)
        u3 = self._buf("u3", (B, H // 2, W // 2, 128), torch.bfloat16)
        _native.check(lib.pty_ws_up2(B, H // 4, W // 4, 128, _p(h3), _p(u3), sp))
        h4 = self._conv_tc(3, u3, B, H // 2, W // 2, skip=h2, keep=True)
        u4 = self._buf("u4", (B, H, W, 64), torch.bfloat16)
        _native.check(lib.pty_ws_up2(B, H // 2, W // 2, 64, _p(h4), _p(u4), sp))
        h5 = self._conv_tc(4, u4, B, H, W, skip=h1, keep=True)
        # the layer inputs the backward pass's im2col reads
        self._fwd_inputs = (x, p1, p2, u3, u4, h5)
        return self._conv_direct(5, h5, B, H, W, last=True)

    def _conv_direct(self, i, x, B, H, W, last=False):
        """Layer i on the CUDA-core direct convolution (the 2-channel first
        and last layers, too narrow for a tensor-core tile): bf16 activation,
        or the FP32 output if last."""
        torch = _torch()
        cin, cout, relu, _ = LAYERS[i]
        if last:
            y = self._buf("y", (B, H, W, cout), torch.float32)
            _native.check(self.lib.pty_ws_conv3x3_direct(B, H, W, cin, cout, _p(x), _p(self.wb[i]), _p(self.b[i]),
                                                         int(relu), None, None, _p(y), self._sp()))
            return y
        out = self._buf("d%d" % i, (B, H, W, cout), torch.bfloat16)
        _native.check(self.lib.pty_ws_conv3x3_direct(B, H, W, cin, cout, _p(x), _p(self.wb[i]), _p(self.b[i]),
                                                     int(relu), None, _p(out), None, self._sp()))
        return out

    def forward_infer(self, x):
        """The forward pass for inference: layers 1-4 (the network's bulk,
        32-128 channels) on the tensor-core convolution, the 2-channel first
        and last layers on the CUDA-core direct convolution; neither writes
        an im2col buffer or keeps anything for a backward pass.  Same result
        as forward() up to FP32 summation order."""
        torch = _torch()
        B, H, W = x.shape[0], self.H, self.W
        lib, sp = self.lib, self._sp()
        h1 = self._conv_direct(0, x, B, H, W)
        p1 = self._buf("p1", (B, H // 2, W // 2, 32), torch.bfloat16)
        _native.check(lib.pty_ws_pool2(B, H, W, 32, _p(h1), _p(p1), sp))
        h2 = self._conv_tc(1, p1, B, H // 2, W // 2)
        p2 = self._buf("p2", (B, H // 4, W // 4, 64), torch.bfloat16)
        _native.check(lib.pty_ws_pool2(B, H // 2, W // 2, 64, _p(h2), _p(p2), sp))
        h3 = self._conv_tc(2, p2, B, H // 4, W // 4)
        u3 = self._buf("u3", (B, H // 2, W // 2, 128), torch.bfloat16)
        _native.check(lib.pty_ws_up2(B, H // 4, W // 4, 128, _p(h3), _p(u3), sp))
        h4 = self._conv_tc(3, u3, B, H // 2, W // 2, skip=h2)
        u4 = self._buf("u4", (B, H, W, 64), torch.bfloat16)
        _native.check(lib.pty_ws_up2(B, H // 2, W // 2, 64, _p(h4), _p(u4), sp))
        h5 = self._conv_tc(4, u4, B, H, W, skip=h1)
        return self._conv_direct(5, h5, B, H, W, last=True)

    def _conv_bwd(self, i, dA, B, H, W, need_dx):
        """dA: gradient (FP32, B x H x W x C_out) at layer i's activation; sets
        the layer's weight and bias gradients, returns the input gradient."""
        torch = _torch()
        cin, cout, relu, _ = LAYERS[i]
        lib, sp = self.lib, self._sp()
        P, K = B * H * W, 9 * cin
        a = self._bufs["a%d" % i] if relu else None
        tc = getattr(self, "_fwd_inputs", None) is not None
        wscr_n = int(lib.pty_ws_wgrad_tc_scratch(B, H, W, cin, cout)) if tc else -1
        if tc and wscr_n < 0:
            # a tensor-core forward pass wrote no im2col buffer: form it now
            col = self._buf("col%d" % i, (P, K), torch.bfloat16)
            _native.check(lib.pty_ws_im2col(B, H, W, cin, _p(self._fwd_inputs[i]), _p(col), sp))
        dZ = self._buf("dz", (P, cout), torch.bfloat16)
        scr = self._buf("actscr", (int(lib.pty_ws_act_bwd_scratch(P, cout)),), torch.float32)
        _native.check(lib.pty_ws_act_bwd(P, cout, _p(dA), _p(a), int(relu), _p(dZ), _p(self.gb[i]),
                                         _p(scr), sp))
        if wscr_n >= 0:
            # wgrad on the tensor cores from channel-major copies of the layer
            # input (three x-shifted) and of dZ; no im2col buffer
            xs = self._buf("xs", (3, cin, P), torch.bfloat16)
            _native.check(lib.pty_ws_shift_transpose(B, H, W, cin, 3, _p(self._fwd_inputs[i]), _p(xs), sp))
            dzt = self._buf("dzt", (cout, P), torch.bfloat16)
            _native.check(lib.pty_ws_shift_transpose(B, H, W, cout, 1, _p(dZ), _p(dzt), sp))
            wscr = self._buf("wscr", (wscr_n,), torch.float32)
            _native.check(lib.pty_ws_wgrad_tc(B, H, W, cin, cout, _p(xs), _p(dzt), _p(self.gw[i]), _p(wscr),
                                              wscr_n, sp))
        else:
            # wgrad: dW[co][k] = sum_p dZ[p][co] col[p][k], split over pixels
            # (about two CTAs per SM: tiles x splits ~ 304)
            tiles = ((cout + 63) // 64) * ((K + 63) // 64)
            splits = max(1, min(512, P // 1024, (304 + tiles - 1) // tiles))
            part = self._buf("wpart", (splits, cout, K), torch.float32)
            col = self._bufs["col%d" % i]
            _native.check(lib.pty_ws_gemm(cout, K, P, _p(dZ), 1, cout, _p(col), K, 1,
                                          _p(self.gw[i]), K, 1, splits, _p(part), sp))
        if not need_dx:
            return None
        if tc:
            # input gradient as a convolution of dZ with the flipped weights:
            # the tensor-core kernel for layers 1-4, the direct one for the
            # 2-channel layer 5; no dcol buffer, no col2im
            wf = self._buf("wf%d" % i, (cin, 9 * cout), torch.bfloat16)
            _native.check(lib.pty_ws_flip_weights(cin, cout, _p(self.wb[i]), _p(wf), sp))
            dX = self._buf("dx%d" % i, (B, H, W, cin), torch.float32)
            if cout < 32:
                _native.check(lib.pty_ws_conv3x3_direct(B, H, W, cout, cin, _p(dZ), _p(wf), _p(self._zero_bias),
                                                        0, None, None, _p(dX), sp))
            else:
                _native.check(lib.pty_ws_conv3x3_tc_f32(B, H, W, cout, cin, _p(dZ), _p(wf), _p(dX), sp))
            return dX
        dcol = self._buf("dcol", (P, K), torch.float32)
        _native.check(lib.pty_ws_gemm(P, K, cout, _p(dZ), cout, 1, _p(self.wb[i]), K, 1,
                                      _p(dcol), K, 1, 1, None, sp))
        dX = self._buf("dx%d" % i, (B, H, W, cin), torch.float32)
        _native.check(lib.pty_ws_col2im(B, H, W, cin, _p(dcol), _p(dX), sp))
        return dX

    def backward(self, dy):
        """dy: (B, H, W, 2) FP32 gradient at the output; fills self.gw / self.gb."""
        torch = _torch()
        if not hasattr(self, "gw"):
            self.gw = [torch.empty_like(w) for w in self.w]
            self.gb = [torch.empty_like(b) for b in self.b]
        B, H, W = dy.shape[0], self.H, self.W
        lib, sp = self.lib, self._sp()
        dh5 = self._conv_bwd(5, dy, B, H, W, True)                  # h5 = a4 + h1
        du4 = self._conv_bwd(4, dh5, B, H, W, True)
        dh4 = self._buf("dh4", (B, H // 2, W // 2, 64), torch.float32)
        _native.check(lib.pty_ws_up2_bwd(B, H // 2, W // 2, 64, _p(du4), _p(dh4), sp))
        du3 = self._conv_bwd(3, dh4, B, H // 2, W // 2, True)       # h4 = a3 + h2
        dh3 = self._buf("dh3", (B, H // 4, W // 4, 128), torch.float32)
        _native.check(lib.pty_ws_up2_bwd(B, H // 4, W // 4, 128, _p(du3), _p(dh3), sp))
        dp2 = self._conv_bwd(2, dh3, B, H // 4, W // 4, True)
        dh2 = self._buf("dh2", (B, H // 2, W // 2, 64), torch.float32)
        _native.check(lib.pty_ws_pool2_bwd(B, H // 2, W // 2, 64, _p(dp2), _p(dh2), sp))
        _native.check(lib.pty_ws_add(dh2.numel(), _p(dh2), _p(dh4), _p(dh2), sp))
        dp1 = self._conv_bwd(1, dh2, B, H // 2, W // 2, True)
        dh1 = self._buf("dh1", (B, H, W, 32), torch.float32)
        _native.check(lib.pty_ws_pool2_bwd(B, H, W, 32, _p(dp1), _p(dh1), sp))
        _native.check(lib.pty_ws_add(dh1.numel(), _p(dh1), _p(dh5), _p(dh1), sp))
        self._conv_bwd(0, dh1, B, H, W, False)

    def loss_grad(self, y, target, weight):
        """Weighted squared error (weights summing to 1) and its gradient; the
        loss is returned as a device scalar tensor (no host sync)."""
        torch = _torch()
        P = y.shape[0] * self.H * self.W
        dy = self._buf("dy", tuple(y.shape), torch.float32)
        parts = self._buf("lparts", (256,), torch.float32)
        _native.check(self.lib.pty_ws_loss(P, _p(y), _p(target), _p(weight), _p(dy), _p(parts),
                                           self._sp()))
        return parts, dy

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        sp = self._sp()
        params = list(zip(self.w, self.wb, self.gw)) + [(b, None, g) for b, g in zip(self.b, self.gb)]
        for (w, wb, g), m, v in zip(params, self.m, self.v):
            _native.check(self.lib.pty_ws_adam(w.numel(), _p(w), _p(wb), _p(g), _p(m), _p(v),
                                               lr, b1, b2, eps, self.step_count, sp))

    def train_step(self, x, target, weight, lr=1e-3, tensor_cores=True):
        """One Adam step on a batch; the forward pass on the tensor cores
        (forward_train) unless tensor_cores is False (forward)."""
        if tensor_cores:
            y = self.forward_train(x)
        else:
            self._fwd_inputs = None
            y = self.forward(x)
        parts, dy = self.loss_grad(y, target, weight)
        self.backward(dy)
        self.adam_step(lr)
        return parts

    # ------------------------------------------------------------ data
    def input_from_intensities(self, plan_h, I, P, phasors, x=None):
        """The network input for the frames of a plan (n frames of H x W): the
        centred intensities I (n, H, W) float32, the probe P (H, W) and
        phasors = probe_phasors(P) (complex64), all device tensors.  Returns
        x (n, H, W, 2) bf16 (written into x when given)."""
        torch = _torch()
        n, H, W = I.shape[0], self.H, self.W
        g = _native.plan_geometry(plan_h)
        # the plan's kernels write all of its frames: the buffers below hold n
        if (g.n_frames, g.N0, g.N1) != (n, H, W):
            raise ValueError("the plan is for %d frames of %d x %d, the intensities hold %s"
                             % (g.n_frames, g.N0, g.N1, tuple(I.shape)))
        lib, sp = self.lib, self._sp()
        if x is None:
            x = torch.empty((n, H, W, 2), dtype=torch.bfloat16, device=self.dev)
        amp = self._buf("amp", (n, H, W), torch.float32)
        _native.check(lib.pty_amp_from_intensity(plan_h, _p(I), 0, _p(amp), sp))
        bp = self._buf("bp", (n, H, W), torch.complex64)
        _native.check(lib.pty_back_project(plan_h, _p(amp), None, _p(phasors), _p(bp), sp))
        _native.check(lib.pty_ws_prep_bp(n, H, W, _p(bp), _p(P), 1, _p(x), sp))
        return x

    def predict_exits(self, I, P, plan_h, batch=256, tensor_cores=True, phasors=None):
        """Exit waves P exp(i phase) (or |P| exp(i phase)) with the predicted
        phases, for the centred intensities I (n, H, W) float32 of the plan's
        frames and the probe P (H, W) complex64, both on the device."""
        torch = _torch()
        n = I.shape[0]
        if phasors is None:
            phasors = probe_phasors(P.cpu().numpy(), self.dev)
        x = self.input_from_intensities(plan_h, I, P, phasors)
        psi = torch.empty((n, self.H, self.W), dtype=torch.complex64, device=self.dev)
        for s in range(0, n, batch):
            e = min(n, s + batch)
            y = self.forward_infer(x[s:e]) if tensor_cores else self.forward(x[s:e])
            _native.check(self.lib.pty_ws_exits(e - s, self.H * self.W, _p(y), _p(P),
                                                int(self.object_phase), _p(psi[s:]), self._sp()))
        return psi


def probe_phasors(P, device):
    """fftshift(exp(i angle(fftn(P)))) as a complex64 device tensor.
    pty_back_project uses the amplitudes in the reference's centred order;
    with these shifted phasors its output is the back-projection with natural
    order amplitudes times (-1)^(row + col), which pty_ws_prep_bp undoes."""
    torch = _torch()
    ph = np.fft.fftshift(np.exp(1j * np.angle(np.fft.fftn(np.asarray(P, np.complex128)))))
    return torch.from_numpy(np.ascontiguousarray(ph.astype(np.complex64))).to(device)


# ---------------------------------------------------------------- training data
def smooth01(rng, shape, sigma=4.0):
    """Gaussian-filtered uniform noise rescaled to [0, 1]."""
    import scipy.ndimage as ndi
    a = ndi.gaussian_filter(rng.random(shape), sigma)
    return (a - a.min()) / (a.max() - a.min())


def random_object(rng, U, V=None, sigma=4.0):
    """amplitude 0.5 + 0.5 s1, phase pi (s2 - 1/2), s1, s2 smooth random
    fields of smoothing width sigma."""
    V = V or U
    return ((0.5 + 0.5 * smooth01(rng, (U, V), sigma))
            * np.exp(1j * np.pi * (smooth01(rng, (U, V), sigma) - 0.5)))


def aperture_probe(N, radius, edge, quad):
    """Circular aperture with a Gaussian edge and quadratic phase quad r^2."""
    y, x = np.mgrid[:N, :N] - N / 2
    r = np.sqrt(x ** 2 + y ** 2)
    amp = np.exp(-np.clip(r - radius, 0, None) ** 2 / (2 * edge ** 2)) * (r < radius + 3 * edge)
    return amp * np.exp(1j * quad * r ** 2)


class _FramePlan:
    """A plan for n frames of N x N in a U x V object (the library's C ABI)."""

    def __init__(self, n, N, U, V, R):
        self.lib = _native.load()
        R64 = np.ascontiguousarray(np.asarray(R)[:, :2], dtype=np.int64)
        self._win_host = np.ascontiguousarray(-R64, dtype=np.int32)   # object window of each frame
        self._win = None
        self.h = ctypes.c_void_p()
        _native.check(self.lib.pty_plan_create(ctypes.byref(_native.Geometry(n, N, N, U, V)),
                                               R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                               ctypes.byref(self.h)))

    def windows(self, device):
        """Each frame's object window start (-R), int32 (n, 2) on the device."""
        if self._win is None:
            self._win = _torch().from_numpy(self._win_host).to(device)
        return self._win

    def close(self):
        if self.h:
            self.lib.pty_plan_destroy(self.h)
            self.h = ctypes.c_void_p()


def make_training_set(net, n_frames, seed=0, frames_per_object=8, batch=32, pad=64, sigma=(4.0, 4.0),
                      photons=None):
    """Frames of random objects (random_object, smoothing width drawn from
    `sigma`) under random probes (aperture radius 24-40 px, edge 4 px,
    quadratic phase 0.001-0.004 rad/px^2) at random positions: the network
    input (the frames' back-projections, input_from_intensities), the
    targets (cos, sin of the object phase under the probe) and weights |P|^2
    scaled so that `batch` frames sum to 1.  With photons = (lo, hi) each
    object's frames get Poisson noise at a photon count per frame drawn
    log-uniformly from that range.  All on the device."""
    torch = _torch()
    N, dev, lib = net.H, net.dev, net.lib
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    n = (n_frames // frames_per_object) * frames_per_object
    x = torch.empty((n, N, N, LAYERS[0][0]), dtype=torch.bfloat16, device=dev)
    t = torch.empty((n, N, N, 2), dtype=torch.float32, device=dev)
    w = torch.empty((n, N, N), dtype=torch.float32, device=dev)
    k = frames_per_object
    I = torch.empty((k, N, N), dtype=torch.float32, device=dev)
    psi = torch.empty((k, N, N), dtype=torch.complex64, device=dev)
    U = N + pad
    sp = net._sp()
    for s in range(0, n, k):
        sg = float(sigma[0]) if sigma[0] == sigma[1] else float(rng.uniform(sigma[0], sigma[1]))
        O = random_object(rng, U, sigma=sg)
        P = aperture_probe(N, rng.uniform(24, 40), 4.0, rng.uniform(0.001, 0.004))
        R = -rng.integers(0, U - N + 1, (k, 2))
        R[0] = 0                                       # the plan's window starts at R.max() = 0
        Od = torch.from_numpy(O.astype(np.complex64)).to(dev)
        Pd = torch.from_numpy(P.astype(np.complex64)).to(dev)
        plan = _FramePlan(k, N, U, U, R)
        try:
            _native.check(lib.pty_intensities(plan.h, _p(Od), _p(Pd), _p(I), sp))
            if photons is not None:
                ph = 10.0 ** rng.uniform(np.log10(photons[0]), np.log10(photons[1]))
                I.copy_(torch.poisson(I * (ph / I.sum(dim=(1, 2), keepdim=True)), generator=gen))
            _native.check(lib.pty_make_exits(plan.h, _p(Od), _p(Pd), _p(psi), sp))
            net.input_from_intensities(plan.h, I, Pd, probe_phasors(P, dev), x[s:s + k])
            wscale = 1.0 / (batch * float(np.sum(np.abs(P) ** 2)))
            _native.check(lib.pty_ws_targets(k, N * N, _p(psi), _p(Pd), int(net.object_phase), wscale,
                                             _p(t[s:]), _p(w[s:]), sp))
            torch.cuda.current_stream(dev).synchronize()
        finally:
            plan.close()
    return x, t, w


def train(net, data, steps, batch=32, lr=1e-3, seed=0, log_every=0):
    """Adam on random contiguous batches of the training set; returns the
    per-step losses (host floats, read once at the end)."""
    torch = _torch()
    x, t, w = data
    n = x.shape[0]
    rng = np.random.default_rng(seed)
    hist = torch.zeros((steps, 256), dtype=torch.float32, device=net.dev)
    for step in range(steps):
        s = int(rng.integers(0, n - batch + 1))
        lr_s = lr * (0.1 if step >= int(0.8 * steps) else 1.0)     # one decay step
        hist[step].copy_(net.train_step(x[s:s + batch], t[s:s + batch], w[s:s + batch], lr_s))
        if log_every and (step + 1) % log_every == 0:
            print("step %d loss %.4f" % (step + 1, float(hist[step].sum().cpu())), flush=True)
    return hist.sum(dim=1, dtype=torch.float64).cpu().numpy().tolist()


def warm_start_object(net, I_dev, P_dev, plan_h, U, V, alpha=1e-10, heat=None, phasors=None, align=0, win=None):
    """The initial object for ERA: the network's exit waves for the centred
    intensities I_dev (n, N, N) float32, stitched by the overlap update
    (psup_O, era.py:336-369) with the probe P_dev on the plan's U x V grid.
    plan_h must be a plan of exactly these n frames of N x N (its kernels
    read n frames of I_dev; a mismatch raises ValueError).  With align > 0
    and win (the frames' object window starts, int32 (n, 2) on the device)
    each frame's phase offset against the stitched object is removed
    (pty_ws_align_phase) and the frames stitched again, align times: a
    frame's far-field data fix its object phase only up to a constant, so
    the network's frames disagree by per-frame offsets.  Returns a complex64
    (U, V) device tensor."""
    torch = _torch()
    g = _native.plan_geometry(plan_h)
    if (g.U, g.V) != (U, V):
        raise ValueError("the plan's object is %d x %d, not %d x %d" % (g.U, g.V, U, V))
    psi = net.predict_exits(I_dev, P_dev, plan_h, phasors=phasors)
    O = torch.empty((U, V), dtype=torch.complex64, device=net.dev)
    if heat is None:
        heat = torch.empty((U, V), dtype=torch.float64, device=net.dev)
    _native.check(net.lib.pty_psup_O(plan_h, _p(psi), _p(P_dev), _p(heat), 1, alpha, _p(O), net._sp()))
    if align > 0 and win is None:
        raise ValueError("align needs the frames' object windows (win)")
    n, N0, N1 = psi.shape
    for _ in range(align):
        _native.check(net.lib.pty_ws_align_phase(n, N0, N1, _p(win), U, V, _p(O), _p(P_dev), _p(psi), net._sp()))
        _native.check(net.lib.pty_psup_O(plan_h, _p(psi), _p(P_dev), _p(heat), 0, alpha, _p(O), net._sp()))
    return O


def initial_object(net, I, R, P, O_shape=None, alpha=1e-10, align=2):
    """The warm start for ``ERA(I, R, P, O, ...)`` on host arrays: centred
    intensities I (n, N, N), scan offsets R (n, 2) and the probe P (N, N),
    as ERA takes them.  R is shifted as ERA's preamble shifts it
    (era.py:504-505, on a copy); the object has ERA's default shape
    (era.py:480-486) unless O_shape is given; the frames' phase offsets are
    aligned `align` times (warm_start_object).  Returns a complex64 host
    array to pass as ERA's O."""
    torch = _torch()
    I = np.asarray(I)
    n, N0, N1 = I.shape
    if (N0, N1) != (net.H, net.W):
        raise ValueError("the network was built for %d x %d frames" % (net.H, net.W))
    R = np.array(R, dtype=np.int64, copy=True)[:, :2]
    R[:, 0] -= R[:, 0].max()
    R[:, 1] -= R[:, 1].max()
    if O_shape is None:
        O_shape = (N0 + int(R[:, 0].max() - R[:, 0].min()), N1 + int(R[:, 1].max() - R[:, 1].min()))
    U, V = O_shape
    plan = _FramePlan(n, N0, U, V, R)
    try:
        I_d = torch.from_numpy(np.ascontiguousarray(I, dtype=np.float32)).to(net.dev)
        P_d = torch.from_numpy(np.ascontiguousarray(P, dtype=np.complex64)).to(net.dev)
        O = warm_start_object(net, I_d, P_d, plan.h, U, V, alpha, align=align, win=plan.windows(net.dev))
        return O.cpu().numpy()
    finally:
        plan.close()


def covering_frames(R, P, frac=0.3, lit=1e-2, spacing=1.0):
    """A subset of a scan's frames that still lights the whole object, for a
    warm start that needs each object pixel seen once, not every time the
    scan revisits it.  R: (n, 2) scan offsets with maximum 0 (the plan's),
    P: the probe (N0, N1).  Host work (set-up, once per scan).

    Frames are taken outermost first (distance of their offset from the
    scan's mean) whenever their offset is at least spacing x r from every
    frame taken, r the radius of the probe's half-maximum intensity disc;
    then, for every
    object pixel the full scan lights (sum of |P|^2 over all frames above
    `lit` of its maximum) where no taken frame's |P|^2 reaches `frac` of the
    best any frame gives it, the frame giving it most is added.  Returns the
    sorted frame indices."""
    R = np.asarray(R, np.int64)[:, :2]
    n = len(R)
    p2 = np.abs(np.asarray(P)) ** 2
    N0, N1 = p2.shape
    U, V = N0 + int(R[:, 0].max() - R[:, 0].min()), N1 + int(R[:, 1].max() - R[:, 1].min())
    heat = np.zeros((U, V))
    best_all = np.zeros((U, V))
    for r0, r1 in R:
        w = (slice(-r0, -r0 + N0), slice(-r1, -r1 + N1))
        heat[w] += p2
        np.maximum(best_all[w], p2, out=best_all[w])
    radius = spacing * np.sqrt(np.count_nonzero(p2 >= 0.5 * p2.max()) / np.pi)
    pos = -R.astype(np.float64)
    order = np.argsort(-np.hypot(*(pos - pos.mean(axis=0)).T), kind="stable")
    taken = np.zeros(n, bool)
    kept = np.empty((0, 2))
    for f in order:
        if len(kept) == 0 or np.min(np.hypot(*(kept - pos[f]).T)) >= radius:
            taken[f] = True
            kept = np.vstack((kept, pos[f]))
    best = np.zeros((U, V))
    for f in np.flatnonzero(taken):
        w = (slice(-R[f, 0], -R[f, 0] + N0), slice(-R[f, 1], -R[f, 1] + N1))
        np.maximum(best[w], p2, out=best[w])
    region = heat > lit * heat.max()
    while True:
        short = np.flatnonzero((region & (best < frac * best_all)).ravel())
        if len(short) == 0:
            break
        u, v = divmod(int(short[0]), V)
        a, b = u + R[:, 0], v + R[:, 1]                 # the pixel in each frame
        inside = (a >= 0) & (a < N0) & (b >= 0) & (b < N1) & ~taken
        cand = np.flatnonzero(inside)
        f = int(cand[np.argmax(p2[a[cand], b[cand]])])
        taken[f] = True
        w = (slice(-R[f, 0], -R[f, 0] + N0), slice(-R[f, 1], -R[f, 1] + N1))
        np.maximum(best[w], p2, out=best[w])
    return np.flatnonzero(taken)


class DownsampledStart:
    """The warm start for frames larger than the network's, each frame seen
    at a coarser real-space sampling: the central net.H x net.W part of
    each centred pattern is the far field of the exit wave low-passed and
    sampled every f = N / net.H pixels (times f^2), and the probe is
    resampled the same way, so their ratio, the object, keeps its scale.
    The coarse frames are stitched at the scan offsets divided by f (to the
    nearest coarse pixel) into a coarse object, which is bilinearly upsampled
    by f onto the full object grid.

    With cover (the default) only the frames covering_frames picks go
    through the network: each object pixel needs one good view for a start,
    and on a dense scan that is a third to a quarter of the frames.  The
    coarse frames' phase offsets are aligned against the stitched object
    `align` times (warm_start_object) before the final stitch.

    Set-up (host work, once per scan: the coarse probe, the frame subset, the
    coarse plan and buffers) happens here; run() is device work plus the
    network's batched inference.  n frames of N x N with N = f net.H, the probe P (N, N)
    (host array), R the plan's scan offsets (n, 2) with maximum 0.
    """

    def __init__(self, net, n, N0, N1, P, R, cover=True, spacing=0.75, graph=True, align=2):
        torch = _torch()
        self.graph = bool(graph)
        self.align = int(align)
        self._graph = self._gkey = self._out = None
        if N0 != N1 or net.H != net.W or N0 % net.H:
            raise ValueError("frames must be square, a multiple of the network's %d x %d" % (net.H, net.W))
        self.net, self.n, self.N, self.M = net, int(n), int(N0), int(net.H)
        self.f = self.N // self.M
        F = np.fft.fftshift(np.fft.fft2(np.asarray(P, np.complex128)))
        o = (self.N - self.M) // 2
        Ps = np.fft.ifft2(np.fft.ifftshift(F[o:o + self.M, o:o + self.M]))
        self.P_s = torch.from_numpy(Ps.astype(np.complex64)).to(net.dev)
        self.phasors = probe_phasors(Ps.astype(np.complex64), net.dev)
        Rs = np.rint(np.asarray(R, np.float64)[:, :2] / self.f).astype(np.int64)
        Rs -= Rs.max(axis=0)
        self.Us = self.M + int(Rs[:, 0].max() - Rs[:, 0].min())
        self.Vs = self.M + int(Rs[:, 1].max() - Rs[:, 1].min())
        # with cover, only a subset of frames that lights every pixel the scan
        # lights (covering_frames) goes through the network
        sel = covering_frames(Rs, Ps, spacing=spacing) if cover else np.arange(self.n)
        self.frames = sel
        self.sel = (torch.from_numpy(sel.astype(np.int32)).to(net.dev) if len(sel) < self.n else None)
        Rsel = Rs[sel]
        Rsel = Rsel - Rsel.max(axis=0)
        self.shift = (Rs[sel].max(axis=0) - Rs.max(axis=0))      # window offset of the subset
        self.Uc = self.M + int(Rsel[:, 0].max() - Rsel[:, 0].min())
        self.Vc = self.M + int(Rsel[:, 1].max() - Rsel[:, 1].min())
        self.plan = _FramePlan(len(sel), self.M, self.Uc, self.Vc, Rsel)
        self.I_s = torch.empty((len(sel), self.M, self.M), dtype=torch.float32, device=net.dev)
        self.heat = torch.empty((self.Uc, self.Vc), dtype=torch.float64, device=net.dev)

    def run(self, I_dev, U, V):
        """The initial object (U, V) complex64 on the device for the centred
        intensities I_dev (n, N, N) float32 on the device.

        With graph (the default) the first call for a given I_dev buffer and
        object shape runs the pass once and captures it as a CUDA graph
        (kernels, tensor maps and buffers fixed); later calls replay it.  The
        returned tensor then belongs to the graph: the next run() overwrites
        it, so copy it to keep it."""
        torch = _torch()
        if tuple(I_dev.shape) != (self.n, self.N, self.N):
            raise ValueError("expected %d frames of %d x %d" % (self.n, self.N, self.N))
        if not self.graph:
            return self._run(I_dev, U, V)
        key = (I_dev.data_ptr(), int(U), int(V))
        if self._gkey != key:
            self._graph = self._gkey = self._out = None
            self._run(I_dev, U, V)                # buffers, kernel attributes, tensor-map encoder
            torch.cuda.current_stream(self.net.dev).synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="thread_local"):
                out = self._run(I_dev, U, V)
            self._graph, self._gkey, self._out = g, key, out
        self._graph.replay()
        return self._out

    def _run(self, I_dev, U, V):
        torch = _torch()
        net, sp = self.net, self.net._sp()
        k = self.I_s.shape[0]
        _native.check(net.lib.pty_ws_crop_center(k, self.N, self.N, self.M, self.M, _p(I_dev), _p(self.sel), 1.0,
                                                 _p(self.I_s), sp))
        O_c = warm_start_object(net, self.I_s, self.P_s, self.plan.h, self.Uc, self.Vc, heat=self.heat,
                                phasors=self.phasors, align=self.align, win=self.plan.windows(net.dev))
        if (self.Uc, self.Vc) != (self.Us, self.Vs):
            # the subset's object window inside the full scan's coarse object
            # (outside it: ones, the default start)
            O_s = torch.ones((self.Us, self.Vs), dtype=torch.complex64, device=net.dev)
            a, b = int(-self.shift[0]), int(-self.shift[1])
            O_s[a:a + self.Uc, b:b + self.Vc] = O_c
        else:
            O_s = O_c
        if self.f == 1:
            return O_s
        O = torch.empty((U, V), dtype=torch.complex64, device=net.dev)
        _native.check(net.lib.pty_ws_upsample_object(self.Us, self.Vs, _p(O_s), U, V, self.f, _p(O), sp))
        return O

    def close(self):
        self._graph = self._gkey = self._out = None
        self.plan.close()
