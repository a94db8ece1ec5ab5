"""The public calls read the caller's intensity array in place when the GPU
reads pageable host memory coherently (pty_device_reads_pageable_memory:
Grace-Blackwell's NVLink-C2C), instead of uploading a copy.  Both paths must
give the same bits: ERA method 6 (the amplitudes and I_norm kernel) and DM
method 1 (the amplitudes kernel, I_norm given), single and double intensities."""
import ctypes

import numpy as np
import pytest

import ptychography_gb300 as pty
from ptychography_gb300 import _engine, _native

pytestmark = pytest.mark.gpu


def _small():
    d = np.load(__file__.rsplit("/", 1)[0] + "/golden/forward_sim.npz")
    return d["I"], d["R"], d["M"], d["P"]


def test_capability_query():
    yes = ctypes.c_int32(-1)
    _native.check(_native.load().pty_device_reads_pageable_memory(ctypes.byref(yes)))
    assert yes.value in (0, 1)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_in_place_read_gives_the_same_bits(dtype, monkeypatch):
    I, R, M, P = _small()
    I = I.astype(dtype)
    out = []
    for enabled in (False, True):
        monkeypatch.setattr(_engine, "HOST_READ_ENABLED", enabled)
        pty.release_plan_cache()
        np.random.seed(5)
        O, Pg, info = pty.ERA(I, R.copy(), P, None, 2, mask=M, method=6)
        O2, info2 = pty.DM(I, R.copy(), P, O, 2, mask=M, method=1)
        out.append((O, Pg, info["eMod"], O2, info2["eMod"]))
    for a, b in zip(*out):
        np.testing.assert_array_equal(np.asarray(a), np.asarray(b))
