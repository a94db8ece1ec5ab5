"""Host side of the drop-in ERA / DM: the reference's preamble, device upload,
one C-ABI call for the whole loop, and the reference's return values.

Host work mirrors ``preamble`` (ptychography/era.py:435-548): the method and
update choice, the dtype rule, the default object of ones, the random initial
probe and background drawn from NumPy's global RNG in the reference's order,
``I_norm``, and the in-place shift of ``R``.  Everything else (amplitudes,
exit waves, FFTs, projections, metrics) runs on the GPU in libptycho_gb300.
Bulk arithmetic is complex64; ``dtype='double'`` only sets the dtype of the
returned arrays.
"""
import ctypes
import math

import numpy as np

from . import _native

_UPDATE = {1: "O", 4: "O", 2: "P", 5: "P", 3: "OP", 6: "OP"}


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("ptychography_gb300 runs on a CUDA GPU; none is available")
    return torch


def choose_method(method, O, P, background):
    """era.py:440-456."""
    if method is None:
        if O is None and P is None:
            method = 3
        elif O is None:
            method = 1
        elif P is None:
            method = 2
        else:
            raise ValueError("method=None needs O or P to be None (era.py:440-449)")
        if background is not None:
            method += 3
    if method not in _UPDATE:
        raise ValueError("method must be one of 1..6, got %r" % (method,))
    return method


def pmod_probe_count(Pmod_probe, iters):
    """Number of leading iterations i with ``i < Pmod_probe`` (era.py:193)."""
    if Pmod_probe is None or Pmod_probe is False:
        return 0
    x = float(Pmod_probe)
    if math.isinf(x):
        return iters if x > 0 else 0
    return max(0, min(iters, int(math.ceil(x))))


class Preamble:
    """Host set-up shared by ERA and DM (era.py:435-548), without exit waves."""

    def __init__(self, I, R, P, O, OP_iters, mask, background, method, dtype):
        I = np.asarray(I)
        if I.ndim != 3:
            raise ValueError("I must be (n_frames, N0, N1)")
        R = np.asarray(R) if not isinstance(R, np.ndarray) else R
        if R.ndim != 2 or R.shape[0] != I.shape[0] or R.shape[1] < 2:
            raise ValueError("R must be (n_frames, 2)")
        self.method = choose_method(method, O, P, background)
        self.update = _UPDATE[self.method]
        if isinstance(OP_iters, (int, np.integer)):
            OP_iters = (int(OP_iters), 1)
        self.OP_iters = (int(OP_iters[0]), int(OP_iters[1]))
        if dtype is None:
            dtype = "single" if I.dtype == np.float32 else "double"
        if dtype not in ("single", "double"):
            raise ValueError("dtype must be None, 'single' or 'double'")
        self.rdt, self.cdt = ((np.float32, np.complex64) if dtype == "single"
                              else (np.float64, np.complex128))
        n, N0, N1 = I.shape
        if O is None:
            O = np.ones((N0 + R[:, 0].max() - R[:, 0].min(), N1 + R[:, 1].max() - R[:, 1].min()),
                        dtype=self.cdt)
        if P is None:
            P = np.random.random(I[0].shape) + 1J * np.random.random(I[0].shape)
        self.P = np.asarray(P).astype(self.cdt)
        self.O = np.asarray(O).astype(self.cdt)
        if self.P.shape != (N0, N1):
            raise ValueError("P must have the frame shape %s" % ((N0, N1),))
        scalar_mask = np.ndim(mask) == 0
        if scalar_mask:
            mask_arr = None
            self.I_norm = float(np.sum(mask * I, dtype=np.float64))
        else:
            mask = np.asarray(mask)
            if mask.shape != (N0, N1):
                raise ValueError("mask must have the frame shape %s" % ((N0, N1),))
            self.I_norm = float(np.sum(mask * I))
            mask_arr = np.ascontiguousarray(np.fft.ifftshift(mask) != 0).astype(np.uint8)
        self.mask = mask_arr
        self.I = I
        R[:, 0] -= R[:, 0].max()                                  # era.py:504-505
        R[:, 1] -= R[:, 1].max()
        self.R = R
        self.n, self.N0, self.N1 = n, N0, N1
        self.background = None
        if self.method in (4, 5, 6):                              # era.py:539-544
            if background is None:
                self.background = (np.random.random((n, N0, N1)).astype(self.rdt) + 0.1).astype(np.float32)
            else:
                b = np.sqrt(np.fft.ifftshift(np.asarray(background, dtype=np.float64)))
                self.background = np.ascontiguousarray(
                    np.broadcast_to(b.astype(np.float32), (n, N0, N1)))
        self.user_background = background
        Pamp = np.fft.fftn(self.P, axes=(-2, -1))                 # era.py:546-547
        self.Pamp = np.sqrt((Pamp.conj() * Pamp).real).astype(np.float32)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def run(kind, I, R, P, O, iters, OP_iters, mask, background, method, Pmod_probe,
        probe_centering, alpha, dtype, full_output, use_graph=True):
    """Run ERA (kind='era') or DM (kind='dm') on the GPU; return the reference's outputs."""
    torch = _torch()
    lib = _native.load()
    pre = Preamble(I, R, P, O, OP_iters, mask, background, method, dtype)
    iters = int(iters)
    dev = torch.device("cuda", torch.cuda.current_device())
    n, N0, N1 = pre.n, pre.N0, pre.N1
    U, V = pre.O.shape

    geom = _native.Geometry(n, N0, N1, U, V)
    R64 = np.ascontiguousarray(pre.R[:, :2], dtype=np.int64)
    plan = ctypes.c_void_p()
    _native.check(lib.pty_plan_create(ctypes.byref(geom),
                                      R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                      ctypes.byref(plan)))
    try:
        stream = torch.cuda.current_stream(dev)
        sp = ctypes.c_void_p(stream.cuda_stream)
        Iin = pre.I
        if Iin.dtype not in (np.float32, np.float64):
            Iin = Iin.astype(np.float64)
        I_d = torch.from_numpy(np.ascontiguousarray(Iin)).to(dev, non_blocking=False)
        amp = torch.empty((n, N0, N1), dtype=torch.float32, device=dev)
        _native.check(lib.pty_amp_from_intensity(plan, _ptr(I_d), int(Iin.dtype == np.float64),
                                                 _ptr(amp), sp))
        del I_d
        O_d = torch.from_numpy(np.ascontiguousarray(pre.O.astype(np.complex64))).to(dev)
        P_d = torch.from_numpy(np.ascontiguousarray(pre.P.astype(np.complex64))).to(dev)
        psi = torch.empty((n, N0, N1), dtype=torch.complex64, device=dev)
        mask_d = torch.from_numpy(pre.mask).to(dev) if pre.mask is not None else None
        bg_d = torch.from_numpy(pre.background).to(dev) if pre.background is not None else None
        npm = pmod_probe_count(Pmod_probe, iters)
        Pamp_d = torch.from_numpy(pre.Pamp).to(dev) if npm > 0 else None
        bmean = torch.zeros((N0, N1), dtype=torch.float32, device=dev) if bg_d is not None else None
        heat = torch.zeros((U, V), dtype=torch.float64, device=dev)
        inten = (torch.empty((n, N0, N1), dtype=torch.float32, device=dev)
                 if full_output and iters > 0 else None)
        emod = torch.zeros(max(iters, 1), dtype=torch.float64, device=dev)
        econ = torch.zeros(max(iters, 1), dtype=torch.float64, device=dev)

        buf = _native.Buffers(_ptr(O_d), _ptr(P_d), _ptr(psi), _ptr(amp), _ptr(mask_d), _ptr(bg_d),
                              _ptr(Pamp_d), _ptr(bmean), _ptr(heat), _ptr(inten), _ptr(emod),
                              _ptr(econ))
        opt = _native.Options(pre.method, pre.OP_iters[0], pre.OP_iters[1], npm,
                              int(bool(probe_centering)), int(bool(use_graph)), float(alpha),
                              pre.I_norm)
        hv = ctypes.c_int32(0)
        fn = lib.pty_era if kind == "era" else lib.pty_dm
        _native.check(fn(plan, ctypes.byref(buf), ctypes.byref(opt), iters, ctypes.byref(hv), sp))
        stream.synchronize()

        O_out = O_d.cpu().numpy().astype(pre.cdt)
        P_out = P_d.cpu().numpy().astype(pre.cdt)
        upd = pre.update
        if not full_output:
            return O_out if upd == "O" else P_out if upd == "P" else (O_out, P_out)
        rt = pre.rdt
        info = {
            "I": inten.cpu().numpy().astype(rt) if inten is not None else None,
            "eMod": [rt(x) for x in emod.cpu().numpy()[:iters]],
            "eCon": [rt(x) for x in econ.cpu().numpy()[:iters]],
            "heatmap": heat.cpu().numpy().astype(rt) if (hv.value and upd != "P") else None,
        }
        if bmean is not None:
            info["background"] = (np.fft.fftshift(bmean.cpu().numpy()) ** 2).astype(rt)
        elif kind == "era" and pre.user_background is not None:
            b = np.asarray(pre.user_background)                   # era.py:311-314
            info["background"] = np.fft.fftshift(b[0] if b.ndim == 3 else b) ** 2
        if upd == "O":
            return O_out, info
        if upd == "P":
            return P_out, info
        return O_out, P_out, info
    finally:
        lib.pty_plan_destroy(plan)
