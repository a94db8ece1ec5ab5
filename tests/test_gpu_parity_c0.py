"""One-step parity at the 128x128 / 100-frame / 320x320 object scale.

The reference's per-iteration contract is checked as a one-step error: the
oracle (FP64 NumPy restatement, pinned to the reference by the golden tests)
runs k iterations, then both the oracle and the GPU apply one more iteration
to that same state; the GPU result must agree within 1e-5 relative (norm-wise)
-- the tolerance stated for FP32 work against the FP64 reference.
"""
import numpy as np
import pytest
import scipy.ndimage as ndi

import ptychography_gb300 as pty
from gpu_util import rel
from oracle import ptycho_oracle as orc

pytestmark = pytest.mark.gpu

ONE_STEP_TOL = 1e-5


def smooth01(rng, shape, sigma=4.0):
    a = ndi.gaussian_filter(rng.random(shape), sigma)
    return (a - a.min()) / (a.max() - a.min())


def c0_problem(seed=0, n_side=10, N=128, U=320):
    """The 100-frame 128x128 noise-free problem: raster step 16, jitter +-2."""
    rng = np.random.default_rng(seed)
    O = (0.5 + 0.5 * smooth01(rng, (U, U))) * np.exp(1j * np.pi * (smooth01(rng, (U, U)) - 0.5))
    y, x = np.mgrid[:N, :N] - N / 2
    r = np.sqrt(x ** 2 + y ** 2)
    edge = np.exp(-np.clip(r - 32, 0, None) ** 2 / (2 * 4.0 ** 2))
    P = edge * (r < 32 + 12) * np.exp(1j * 0.002 * r ** 2)
    pos = np.arange(n_side) * 16 + 16
    R = -np.stack(np.meshgrid(pos, pos, indexing="ij"), -1).reshape(-1, 2)
    R = R + rng.integers(-2, 3, R.shape)
    R = np.minimum(R, 0)
    R = np.maximum(R, -(U - N))
    ex = orc.make_exits(O, P, R)
    I = np.fft.fftshift(np.abs(np.fft.fft2(ex)) ** 2, axes=(-2, -1))
    return I, R, P, O


@pytest.fixture(scope="module")
def c0():
    return c0_problem()


def test_era_m1_one_step(c0):
    I, R, P, O_true = c0
    M = np.ones(I.shape[1:], bool)
    k = 3
    O_k, _ = orc.ERA(I, R.copy(), P, None, k, mask=M, method=1, dtype="double")
    O_k1, info_o = orc.ERA(I, R.copy(), P, O_k, 1, mask=M, method=1, dtype="double")
    O_g, info_g = pty.ERA(I, R.copy(), P, O_k, 1, mask=M, method=1, dtype="double")
    assert rel(O_g, O_k1) < ONE_STEP_TOL
    assert info_g["eMod"][0] == pytest.approx(info_o["eMod"][0], rel=ONE_STEP_TOL)
    assert info_g["eCon"][0] == pytest.approx(info_o["eCon"][0], rel=1e-4)


def test_dm_m3_one_step(c0):
    I, R, P, O_true = c0
    M = np.ones(I.shape[1:], bool)
    P0 = P * 0.95
    O_k, P_k, _ = orc.DM(I, R.copy(), P0, None, 2, mask=M, method=3, dtype="double")
    O_o, P_o, info_o = orc.DM(I, R.copy(), P_k, O_k, 1, mask=M, method=3, dtype="double")
    O_g, P_g, info_g = pty.DM(I, R.copy(), P_k, O_k, 1, mask=M, method=3, dtype="double")
    assert rel(O_g, O_o) < ONE_STEP_TOL
    assert rel(P_g, P_o) < ONE_STEP_TOL
    assert info_g["eMod"][0] == pytest.approx(info_o["eMod"][0], rel=ONE_STEP_TOL)


def test_era_m1_trajectory(c0):
    """Ten GPU iterations from ones track the FP64 oracle (drift reported, bounded)."""
    I, R, P, O_true = c0
    M = np.ones(I.shape[1:], bool)
    O_o, info_o = orc.ERA(I, R.copy(), P, None, 10, mask=M, method=1, dtype="double")
    O_g, info_g = pty.ERA(I, R.copy(), P, None, 10, mask=M, method=1, dtype="single")
    assert rel(O_g, O_o) < 1e-4
    np.testing.assert_allclose(info_g["eMod"], info_o["eMod"], rtol=1e-4)
