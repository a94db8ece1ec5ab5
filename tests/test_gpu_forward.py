"""forward_sim on the GPU against the oracle's restatement of forward_models.py."""
import os

import numpy as np
import pytest

import ptychography_gb300 as pty
from gpu_util import rel
from oracle import ptycho_oracle as orc

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_forward_sim_matches_reference_fixture():
    d = np.load(os.path.join(GOLD, "forward_sim.npz"))
    np.random.seed(int(d["seed"]))
    I, R, M, P, O, B = pty.forward_sim(shape_P=(32, 32), A=9, defocus=0.02, photons_pupil=100.0,
                                       ny=3, nx=3, random_offset=3, background=2, mask=12,
                                       counting_statistics=False, O=d["O"])
    assert np.array_equal(R, d["R"]) and np.array_equal(M, d["M"]) and np.array_equal(B, d["B"])
    np.testing.assert_allclose(P, d["P"], atol=1e-14)
    assert I.dtype == np.float64
    assert rel(I, d["I"]) < 2e-6


def test_forward_sim_rect_default_shape():
    d = np.load(os.path.join(GOLD, "forward_sim_rect.npz"))
    np.random.seed(int(d["seed"]))
    I, R, M, P, O, B = pty.forward_sim(shape_P=(32, 64), A=10, defocus=0.01, photons_pupil=50.0,
                                       ny=3, nx=2, random_offset=4, background=3, mask=8,
                                       counting_statistics=True, O=d["O"])
    assert I.dtype == np.int64
    assert np.array_equal(R, d["R"]) and np.array_equal(M, d["M"])
    # Poisson draws of FP32 intensities agree with the FP64 ones except at most
    # where lam sits on a sampling boundary
    assert np.mean(I == d["I"]) > 0.999


def test_back_projection_matches_reference():
    d = np.load(os.path.join(GOLD, "back_projection.npz"))
    p = np.load(os.path.join(GOLD, "forward_sim.npz"))
    Rc = p["R"].copy()
    O, info = pty.Back_projection(p["I"], Rc, d["P"], None, mask=p["M"])
    assert np.array_equal(Rc, d["R_after"])
    assert rel(info["exits"], d["exits"]) < 2e-6
    assert rel(info["heatmap"], d["heatmap"]) < 1e-7
    assert rel(O, d["O"]) < 2e-6
