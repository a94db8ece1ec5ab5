"""Drop-in ``Back_projection`` (ptychography/back_projection.py:4-88) on the GPU.

Each frame's exit wave is taken as ``ifftn(mask * sqrt(I) * exp(i angle(fftn(P))))``
(the detector phases are assumed to be those of the probe) and the object is the
overlap projection of those waves.  The reference calls ``era.psup_O_1``, which
does not exist; the object update it names is ``psup_O`` (era.py:336-369), used
here.  As in the reference, ``sqrt(I)`` and ``mask`` enter in the detector's
centred order against the unshifted ``fftn(P)`` phases, ``R`` is shifted in
place, and ``info`` holds ``'exits'`` and ``'heatmap'``.
"""
import ctypes

import numpy as np

from . import _native


def Back_projection(I, R, P, O, mask=1, alpha=1.0e-10, full_output=True):
    """Back-project the diffraction amplitudes with the probe's far-field phases."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("ptychography_gb300 runs on a CUDA GPU; none is available")
    lib = _native.load()
    I = np.asarray(I)
    n, N0, N1 = I.shape
    P = np.asarray(P)
    if O is None:                                           # back_projection.py:61-67
        O = np.ones((N0 + R[:, 0].max() - R[:, 0].min(), N1 + R[:, 1].max() - R[:, 1].min()),
                    dtype=P.dtype)
    O = np.asarray(O)
    R[:, 0] -= R[:, 0].max()                                # back_projection.py:70-71
    R[:, 1] -= R[:, 1].max()
    U, V = O.shape
    phase = np.exp(1J * np.angle(np.fft.fftn(P))).astype(np.complex64)
    dev = torch.device("cuda", torch.cuda.current_device())
    geom = _native.Geometry(n, N0, N1, U, V)
    R64 = np.ascontiguousarray(R[:, :2], dtype=np.int64)
    plan = ctypes.c_void_p()
    _native.check(lib.pty_plan_create(ctypes.byref(geom),
                                      R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                      ctypes.byref(plan)))
    try:
        p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        sp = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        Iin = I if I.dtype in (np.float32, np.float64) else I.astype(np.float64)
        I_d = torch.from_numpy(np.ascontiguousarray(Iin)).to(dev)
        amp = torch.empty((n, N0, N1), dtype=torch.float32, device=dev)
        _native.check(lib.pty_amp_from_intensity(plan, p(I_d), int(Iin.dtype == np.float64),
                                                 p(amp), sp))
        del I_d
        mask_d = None
        if np.ndim(mask) != 0:
            mask_d = torch.from_numpy(np.ascontiguousarray(
                np.fft.ifftshift(np.asarray(mask) != 0)).astype(np.uint8)).to(dev)
        ph_d = torch.from_numpy(phase).to(dev)
        exits = torch.empty((n, N0, N1), dtype=torch.complex64, device=dev)
        _native.check(lib.pty_back_project(plan, p(amp), p(mask_d), p(ph_d), p(exits), sp))
        P_d = torch.from_numpy(np.ascontiguousarray(P.astype(np.complex64))).to(dev)
        heat = torch.empty((U, V), dtype=torch.float64, device=dev)
        O_d = torch.empty((U, V), dtype=torch.complex64, device=dev)
        _native.check(lib.pty_psup_O(plan, p(exits), p(P_d), p(heat), 1, float(alpha), p(O_d), sp))
        torch.cuda.current_stream(dev).synchronize()
        O_out = O_d.cpu().numpy().astype(np.result_type(P.dtype, np.complex64))
        if not full_output:
            return O_out
        info = {"exits": exits.cpu().numpy(), "heatmap": heat.cpu().numpy().astype(P.real.dtype)}
        return O_out, info
    finally:
        lib.pty_plan_destroy(plan)
