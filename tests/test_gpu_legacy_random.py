"""The random initial background drawn on the device (pty_legacy_random_background)
equals NumPy's host draw bit for bit and leaves NumPy's global generator in the
same state.  Draws above 2^17 words run as parallel segments started by the
jump-ahead (37 x 128^2: 10 segments, 33 x 256^2: 33, 2 x 512^2: 8).  (ERA /
DM runs of methods 4 and 6 from a random background, which now draw it on the
device, are compared with the reference's own recorded runs in test_gpu_runs.)"""
import numpy as np
import pytest
import torch

from ptychography_gb300 import _engine, _native
from gpu_util import dev, stream

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rdt", [np.float32, np.float64])
@pytest.mark.parametrize("seed,skip,shape", [(0, 0, (3, 32, 32)), (5, 7, (4, 64, 64)),
                                             (9, 311, (1, 16, 16)), (2, 623, (37, 128, 128)),
                                             (17, 100, (33, 256, 256)), (4, 0, (2, 512, 512))])
def test_device_background_matches_host(rdt, seed, skip, shape):
    lib = _native.load()
    np.random.seed(seed)
    np.random.random(skip)
    st0 = np.random.get_state()
    ref = (np.random.random(shape).astype(rdt) + 0.1).astype(np.float32)
    after = np.random.get_state()
    np.random.set_state(st0)
    out = torch.empty(shape, dtype=torch.float32, device=dev())
    _engine.device_random_background(lib, out, rdt, stream())
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    now = np.random.get_state()
    assert now[2] == after[2] and now[3] == after[3]
    np.testing.assert_array_equal(now[1], after[1])


def test_next_draw_continues_stream():
    lib = _native.load()
    np.random.seed(21)
    st0 = np.random.get_state()
    np.random.random((2, 48, 48))
    want = np.random.random(10)
    np.random.set_state(st0)
    out = torch.empty((2, 48, 48), dtype=torch.float32, device=dev())
    _engine.device_random_background(lib, out, np.float32, stream())
    np.testing.assert_array_equal(np.random.random(10), want)


def test_caller_scratch_matches_internal():
    lib = _native.load()
    shape = (3, 64, 64)
    np.random.seed(44)
    st0 = np.random.get_state()
    a = torch.empty(shape, dtype=torch.float32, device=dev())
    _engine.device_random_background(lib, a, np.float32, stream())
    after = np.random.get_state()
    np.random.set_state(st0)
    import ctypes
    key = np.ascontiguousarray(st0[1], dtype=np.uint32)
    words = lib.pty_legacy_random_scratch_words(int(st0[2]), a.numel())
    scratch = torch.empty(int(words), dtype=torch.int32, device=dev())
    b = torch.empty_like(a)
    key_out = np.empty(624, dtype=np.uint32)
    pos = ctypes.c_int32(0)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    _native.check(lib.pty_legacy_random_background(
        key.ctypes.data_as(u32p), int(st0[2]), a.numel(), 0, ctypes.c_void_p(b.data_ptr()),
        ctypes.c_void_p(scratch.data_ptr()), key_out.ctypes.data_as(u32p), ctypes.byref(pos),
        stream()))
    np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
    np.testing.assert_array_equal(key_out, after[1])
    assert pos.value == after[2]
    assert lib.pty_legacy_random_scratch_words(625, 1) == -1
