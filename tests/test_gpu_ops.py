"""Each C-ABI operator against the reference's own outputs (tests/golden/ops.npz).

The fixture was recorded in FP64 by the reference; the engine computes in
complex64, so the bound is FP32 rounding of a 32x64 FFT round trip: 2e-6
relative (norm-wise) for waves, 1e-6 for the gathers, 1e-5 for error sums.
"""
import os

import numpy as np
import pytest
import torch

from gpu_util import Plan, ptr, rel, to_dev

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ops.npz")


@pytest.fixture(scope="module")
def ops():
    d = np.load(GOLD)
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="module")
def plan(ops):
    n, N0, N1 = ops["exits"].shape
    U, V = ops["O"].shape
    p = Plan(n, N0, N1, U, V, ops["R"])
    yield p
    p.close()


def test_make_exits(ops, plan):
    O, P = to_dev(ops["O"], np.complex64), to_dev(ops["P"], np.complex64)
    psi = torch.empty(ops["exits"].shape, dtype=torch.complex64, device=O.device)
    plan.call("pty_make_exits", ptr(O), ptr(P), ptr(psi))
    assert rel(psi.cpu().numpy(), ops["make_exits"]) < 1e-6


def test_pmod_1(ops, plan):
    psi = to_dev(ops["exits"], np.complex64)
    amp = to_dev(ops["amp"], np.float32)
    mask = to_dev(ops["mask"], np.uint8)
    e = torch.zeros(1, dtype=torch.float64, device=psi.device)
    plan.call("pty_pmod_1", ptr(amp), ptr(psi), ptr(mask), 1e-10, ptr(e))
    assert rel(psi.cpu().numpy(), ops["pmod_1"]) < 2e-6
    assert float(e.cpu()[0]) == pytest.approx(float(ops["pmod_1_eMod"]), rel=1e-5)


def test_pmod_7(ops, plan):
    psi = to_dev(ops["exits"], np.complex64)
    amp = to_dev(ops["amp"], np.float32)
    bg = to_dev(ops["bg"], np.float32)
    mask = to_dev(ops["mask"], np.uint8)
    e = torch.zeros(1, dtype=torch.float64, device=psi.device)
    plan.call("pty_pmod_7", ptr(amp), ptr(bg), ptr(psi), ptr(mask), 1e-10, ptr(e))
    assert rel(psi.cpu().numpy(), ops["pmod_7"]) < 2e-6
    assert rel(bg.cpu().numpy(), ops["pmod_7_bg"]) < 2e-6
    assert float(e.cpu()[0]) == pytest.approx(float(ops["pmod_7_eMod"]), rel=1e-5)


def test_Pmod_P(ops, plan):
    P = to_dev(ops["P"], np.complex64)
    Pamp = to_dev(ops["Pamp"], np.float32)
    mask = to_dev(ops["mask"], np.uint8)
    plan.call("pty_Pmod_P", ptr(Pamp), ptr(P), ptr(mask), 1e-10)
    assert rel(P.cpu().numpy(), ops["Pmod_P"]) < 2e-6


def test_psup_O_and_heatmap(ops, plan):
    psi = to_dev(ops["exits"], np.complex64)
    P = to_dev(ops["P"], np.complex64)
    U, V = ops["O"].shape
    heat = torch.zeros((U, V), dtype=torch.float64, device=psi.device)
    O = torch.empty((U, V), dtype=torch.complex64, device=psi.device)
    plan.call("pty_psup_O", ptr(psi), ptr(P), ptr(heat), 1, 1e-10, ptr(O))
    assert rel(heat.cpu().numpy(), ops["P_heatmap"]) < 1e-7
    assert rel(O.cpu().numpy(), ops["psup_O"]) < 1e-6
    heat2 = torch.zeros_like(heat)
    plan.call("pty_make_P_heatmap", ptr(P), ptr(heat2))
    assert torch.equal(heat, heat2)


def test_psup_P_and_heatmap(ops, plan):
    psi = to_dev(ops["exits"], np.complex64)
    O = to_dev(ops["O"], np.complex64)
    N0, N1 = ops["P"].shape
    heat = torch.zeros((N0, N1), dtype=torch.float64, device=psi.device)
    P = torch.empty((N0, N1), dtype=torch.complex64, device=psi.device)
    plan.call("pty_psup_P", ptr(psi), ptr(O), ptr(heat), 1, 1e-10, ptr(P))
    assert rel(heat.cpu().numpy(), ops["O_heatmap"]) < 1e-7
    assert rel(P.cpu().numpy(), ops["psup_P"]) < 1e-6
    heat2 = torch.zeros_like(heat)
    plan.call("pty_make_O_heatmap", ptr(O), ptr(heat2))
    assert rel(heat2.cpu().numpy(), ops["O_heatmap"]) < 1e-7


def test_model_error_1(ops, plan):
    psi = to_dev(ops["exits"], np.complex64)
    amp = to_dev(ops["amp"], np.float32)
    mask = to_dev(ops["mask"], np.uint8)
    bg = to_dev(ops["bg"], np.float32)
    e = torch.zeros(1, dtype=torch.float64, device=psi.device)
    plan.call("pty_model_error_1", ptr(amp), ptr(psi), ptr(mask), None, 0, ptr(e))
    assert float(e.cpu()[0]) == pytest.approx(float(ops["model_error_1_nobg"]), rel=1e-5)
    plan.call("pty_model_error_1", ptr(amp), ptr(psi), ptr(mask), ptr(bg), 1, ptr(e))
    assert float(e.cpu()[0]) == pytest.approx(float(ops["model_error_1"]), rel=1e-5)


def test_background_mean(ops, plan):
    bg = to_dev(ops["bg"], np.float32)
    m = torch.empty(ops["bg"].shape[1:], dtype=torch.float32, device=bg.device)
    plan.call("pty_background_mean", ptr(bg), ptr(m))
    np.testing.assert_allclose(m.cpu().numpy(), ops["bg"].mean(axis=0), rtol=1e-6)


def test_amp_from_intensity(ops, plan):
    I = np.abs(ops["amp"]) ** 2
    Ic = np.fft.fftshift(I, axes=(-2, -1))        # centred, as a detector records it
    for dt, isd in ((np.float32, 0), (np.float64, 1)):
        Id = to_dev(Ic, dt)
        amp = torch.empty(I.shape, dtype=torch.float32, device=Id.device)
        plan.call("pty_amp_from_intensity", ptr(Id), isd, ptr(amp))
        np.testing.assert_allclose(amp.cpu().numpy(),
                                   np.fft.ifftshift(np.sqrt(Ic), axes=(-2, -1)), rtol=2e-7)
