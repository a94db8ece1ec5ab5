"""Edge cases on every supported frame shape, against the oracle: a single
frame whose window is the whole object (R = 0, O the probe's size), and two
frames at opposite corners of a just-large-enough object.  Exercises one-entry
tile lists, single-chunk probe gathers and windows on the object's edges."""
import numpy as np
import pytest

import ptychography_gb300 as pty
from gpu_util import rel
from oracle import ptycho_oracle as orc

pytestmark = pytest.mark.gpu

SHAPES = [(32, 32), (64, 64), (32, 64), (128, 128), (192, 192), (256, 256), (512, 512)]


def problem(N0, N1, R, seed):
    rng = np.random.default_rng(seed)
    U = N0 - R[:, 0].min()
    V = N1 - R[:, 1].min()
    O = (0.6 + 0.4 * rng.random((U, V))) * np.exp(1j * rng.random((U, V)))
    y, x = np.mgrid[:N0, :N1]
    P = np.exp(-((y - N0 / 2) ** 2 + (x - N1 / 2) ** 2) / (2 * (min(N0, N1) / 5) ** 2)) + 0j
    ex = orc.make_exits(O, P, R)
    I = np.fft.fftshift(np.abs(np.fft.fft2(ex)) ** 2, axes=(-2, -1))
    O0 = O * (1 + 0.05 * rng.standard_normal(O.shape))
    return I, O0, P * np.exp(0.2j)


@pytest.mark.parametrize("N0,N1", SHAPES)
@pytest.mark.parametrize("frames", [1, 2])
def test_edge_scans(N0, N1, frames):
    R = np.zeros((1, 2), np.int64) if frames == 1 else np.array([[0, 0], [-8, -8]], np.int64)
    I, O0, P0 = problem(N0, N1, R, N0 + frames)
    # an explicit mask: the reference's scalar mask=1 fails in its preamble's
    # ifftshift under current NumPy (era.py:499), and the oracle follows it
    M = np.ones((N0, N1), bool)
    for method in (1, 3):
        want = orc.ERA(I, R.copy(), P0, O0, 2, mask=M, method=method, dtype="double")
        got = pty.ERA(I, R.copy(), P0, O0, 2, mask=M, method=method, dtype="double")
        assert rel(got[0], want[0]) < 2e-5, (method, "O")
        if method == 3:
            assert rel(got[1], want[1]) < 2e-5, (method, "P")
        # one frame determines O exactly: eMod then falls to the FP32 rounding
        # floor (~1e-7, against ~1e-8 in FP64), hence the absolute term
        np.testing.assert_allclose(got[-1]["eMod"], want[-1]["eMod"], rtol=2e-5, atol=1e-6)
