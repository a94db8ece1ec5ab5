"""The random initial background drawn on the device (pty_legacy_random_background)
equals NumPy's host draw bit for bit and leaves NumPy's global generator in the
same state.  (ERA / DM runs of methods 4 and 6 from a random background, which
now draw it on the device, are compared with the reference's own recorded runs
in test_gpu_runs.)"""
import numpy as np
import pytest
import torch

from ptychography_gb300 import _engine, _native
from gpu_util import dev, stream

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rdt", [np.float32, np.float64])
@pytest.mark.parametrize("seed,skip,shape", [(0, 0, (3, 32, 32)), (5, 7, (4, 64, 64)),
                                             (9, 311, (1, 16, 16)), (2, 623, (37, 128, 128))])
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
