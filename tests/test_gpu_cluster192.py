"""192x192 frames: the 2-CTA cluster kernel (radix-3 line codelets) against the oracle.

Operators on random data must match to FP32 rounding of a 192^2 FFT round trip
(3e-6 relative); one ERA / DM method-6 step on a small 192^2 problem with
background, Poisson noise and a beamstop mask must stay within 1e-5 relative.
"""
import numpy as np
import pytest
import torch

import ptychography_gb300 as pty
from gpu_util import Plan, ptr, rel, to_dev
from oracle import ptycho_oracle as orc
from test_gpu_parity_c0 import smooth01

pytestmark = pytest.mark.gpu
N = 192


@pytest.fixture(scope="module")
def rnd():
    rng = np.random.default_rng(192)
    n, U, V = 3, 240, 264
    R = np.stack([-rng.integers(0, U - N + 1, n), -rng.integers(0, V - N + 1, n)], 1)
    c = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)  # noqa: E731
    return dict(n=n, U=U, V=V, R=R, O=c(U, V), P=c(N, N), ex=c(n, N, N),
                amp=np.abs(rng.standard_normal((n, N, N))) * 50,
                bg=np.abs(rng.standard_normal((n, N, N))), mask=rng.random((N, N)) > 0.05)


@pytest.fixture(scope="module")
def plan(rnd):
    p = Plan(rnd["n"], N, N, rnd["U"], rnd["V"], rnd["R"])
    yield p
    p.close()


def test_pmod_1_192(rnd, plan):
    psi = to_dev(rnd["ex"], np.complex64)
    amp, mask = to_dev(rnd["amp"], np.float32), to_dev(rnd["mask"], np.uint8)
    e = torch.zeros(1, dtype=torch.float64, device=psi.device)
    plan.call("pty_pmod_1", ptr(amp), ptr(psi), ptr(mask), 1e-10, ptr(e))
    ref, em = orc.pmod_1(rnd["amp"], rnd["ex"].copy(), rnd["mask"], 1e-10, True)
    assert rel(psi.cpu().numpy(), ref) < 3e-6
    assert float(e.cpu()[0]) == pytest.approx(em, rel=1e-5)


def test_pmod_7_192(rnd, plan):
    psi = to_dev(rnd["ex"], np.complex64)
    amp, mask = to_dev(rnd["amp"], np.float32), to_dev(rnd["mask"], np.uint8)
    bg = to_dev(rnd["bg"], np.float32)
    e = torch.zeros(1, dtype=torch.float64, device=psi.device)
    plan.call("pty_pmod_7", ptr(amp), ptr(bg), ptr(psi), ptr(mask), 1e-10, ptr(e))
    ref, bref, em = orc.pmod_7(rnd["amp"], rnd["bg"].copy(), rnd["ex"].copy(), rnd["mask"], 1e-10, True)
    assert rel(psi.cpu().numpy(), ref) < 3e-6
    assert rel(bg.cpu().numpy(), bref) < 1e-5
    assert float(e.cpu()[0]) == pytest.approx(em, rel=1e-5)


def test_intensities_and_model_error_192(rnd, plan):
    O, P = to_dev(rnd["O"], np.complex64), to_dev(rnd["P"], np.complex64)
    I = torch.empty((rnd["n"], N, N), dtype=torch.float32, device=O.device)
    plan.call("pty_intensities", ptr(O), ptr(P), ptr(I))
    ex = orc.make_exits(rnd["O"], rnd["P"], rnd["R"])
    Iref = np.fft.fftshift(np.abs(np.fft.fft2(ex)) ** 2, axes=(-2, -1))
    assert rel(I.cpu().numpy(), Iref) < 3e-6
    psi = to_dev(rnd["ex"], np.complex64)
    amp, mask = to_dev(rnd["amp"], np.float32), to_dev(rnd["mask"], np.uint8)
    bg0 = to_dev(rnd["bg"][0], np.float32)
    e = torch.zeros(1, dtype=torch.float64, device=O.device)
    plan.call("pty_model_error_1", ptr(amp), ptr(psi), ptr(mask), ptr(bg0), 0, ptr(e))
    em = orc.model_error_1(rnd["amp"], rnd["ex"], rnd["mask"], rnd["bg"][0])
    assert float(e.cpu()[0]) == pytest.approx(em, rel=1e-5)


def small_problem(N, seed=1, side=3, step=None):
    """A side^2-frame problem of N^2 frames: background, Poisson noise, beamstop."""
    rng = np.random.default_rng(seed)
    step = step or N // 8
    U = N + step * (side - 1) + 8
    O = (0.5 + 0.5 * smooth01(rng, (U, U))) * np.exp(1j * np.pi * (smooth01(rng, (U, U)) - 0.5))
    y, x = np.mgrid[:N, :N] - N / 2
    r = np.sqrt(x ** 2 + y ** 2)
    P = (np.exp(-np.clip(r - N / 4, 0, None) ** 2 / 32.0) * (r < N * 0.34)
         * np.exp(1j * 0.0005 * r ** 2))
    pos = np.arange(side) * step + 4
    R = -np.stack(np.meshgrid(pos, pos, indexing="ij"), -1).reshape(-1, 2)
    R = np.clip(R + rng.integers(-3, 4, R.shape), -(U - N), 0)
    ex = orc.make_exits(O, P, R)
    I = np.abs(np.fft.fft2(ex)) ** 2
    blob = np.exp(-((x ** 2 + y ** 2) / (2 * (N / 6.0) ** 2)))
    I = I + 0.01 * I.mean() * np.fft.ifftshift(blob)
    I = np.fft.fftshift(rng.poisson(I * (1e6 / I.sum(axis=(1, 2), keepdims=True))), axes=(-2, -1))
    M = np.ones((N, N), bool)
    M[r < N / 20] = False
    M[rng.random((N, N)) < 0.005] = False
    return I.astype(np.float32), R, P, O, M


@pytest.fixture(scope="module")
def prob192():
    return small_problem(N, seed=3, side=4)


@pytest.mark.parametrize("kind", ["era", "dm"])
def test_m6_one_step_192(prob192, kind):
    I, R, P, O, M = prob192
    np.random.seed(9)
    O_k, P_k, info = orc.ERA(I, R.copy(), P * np.exp(0.1j), None, 2, mask=M, method=6, dtype="double")
    b = info["background"]
    fo, fg = (orc.ERA, pty.ERA) if kind == "era" else (orc.DM, pty.DM)
    O_o, P_o, io = fo(I, R.copy(), P_k, O_k, 1, mask=M, method=6, background=b, dtype="double")
    O_g, P_g, ig = fg(I, R.copy(), P_k, O_k, 1, mask=M, method=6, background=b, dtype="double")
    assert rel(O_g, O_o) < 1e-5 and rel(P_g, P_o) < 1e-5
    assert ig["eMod"][0] == pytest.approx(io["eMod"][0], rel=1e-5)
