"""Helpers for the GPU tests: device tensors and C-ABI calls on a plan."""
import ctypes

import numpy as np
import torch

from ptychography_gb300 import _native


def dev():
    return torch.device("cuda", 0)


def to_dev(a, dtype=None):
    a = np.ascontiguousarray(a if dtype is None else a.astype(dtype))
    return torch.from_numpy(a).to(dev())


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream(dev()).cuda_stream)


class Plan:
    def __init__(self, n, N0, N1, U, V, R):
        self.lib = _native.load()
        self.geom = _native.Geometry(n, N0, N1, U, V)
        R64 = np.ascontiguousarray(np.asarray(R)[:, :2], dtype=np.int64)
        self.h = ctypes.c_void_p()
        _native.check(self.lib.pty_plan_create(
            ctypes.byref(self.geom), R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            ctypes.byref(self.h)))

    def call(self, name, *args):
        _native.check(getattr(self.lib, name)(self.h, *args, stream()))
        torch.cuda.synchronize()

    def close(self):
        self.lib.pty_plan_destroy(self.h)


def rel(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))
