"""512x512 frames: the 16-CTA cluster kernel against the oracle.

Operators on random data (FP32 rounding of a 512^2 FFT round trip: 4e-6
relative), and one ERA / DM iteration (method 6: object, probe, background) on an
8-frame 512^2 problem within 1e-5 relative of the FP64 oracle.
"""
import numpy as np
import pytest
import torch

import ptychography_gb300 as pty
from gpu_util import Plan, ptr, rel, to_dev
from oracle import ptycho_oracle as orc
from test_gpu_parity_c0 import smooth01

pytestmark = pytest.mark.gpu
N = 512


@pytest.fixture(scope="module")
def rnd():
    rng = np.random.default_rng(512)
    n, U, V = 2, 560, 544
    R = np.stack([-rng.integers(0, U - N + 1, n), -rng.integers(0, V - N + 1, n)], 1)
    c = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)  # noqa: E731
    return dict(n=n, U=U, V=V, R=R, O=c(U, V), P=c(N, N), ex=c(n, N, N),
                amp=np.abs(rng.standard_normal((n, N, N))) * 80,
                bg=np.abs(rng.standard_normal((n, N, N))), mask=rng.random((N, N)) > 0.05)


@pytest.fixture(scope="module")
def plan(rnd):
    p = Plan(rnd["n"], N, N, rnd["U"], rnd["V"], rnd["R"])
    yield p
    p.close()


def test_pmod_1_512(rnd, plan):
    psi = to_dev(rnd["ex"], np.complex64)
    amp, mask = to_dev(rnd["amp"], np.float32), to_dev(rnd["mask"], np.uint8)
    e = torch.zeros(1, dtype=torch.float64, device=psi.device)
    plan.call("pty_pmod_1", ptr(amp), ptr(psi), ptr(mask), 1e-10, ptr(e))
    ref, em = orc.pmod_1(rnd["amp"], rnd["ex"].copy(), rnd["mask"], 1e-10, True)
    assert rel(psi.cpu().numpy(), ref) < 4e-6
    assert float(e.cpu()[0]) == pytest.approx(em, rel=1e-5)


def test_pmod_7_and_intensities_512(rnd, plan):
    psi = to_dev(rnd["ex"], np.complex64)
    amp, mask = to_dev(rnd["amp"], np.float32), to_dev(rnd["mask"], np.uint8)
    bg = to_dev(rnd["bg"], np.float32)
    plan.call("pty_pmod_7", ptr(amp), ptr(bg), ptr(psi), ptr(mask), 1e-10, None)
    ref, bref = orc.pmod_7(rnd["amp"], rnd["bg"].copy(), rnd["ex"].copy(), rnd["mask"], 1e-10)
    assert rel(psi.cpu().numpy(), ref) < 4e-6
    # b * f weights the small-|F| pixels, whose FP32 error grows with the transform size
    assert rel(bg.cpu().numpy(), bref) < 2e-5
    O, P = to_dev(rnd["O"], np.complex64), to_dev(rnd["P"], np.complex64)
    I = torch.empty((rnd["n"], N, N), dtype=torch.float32, device=O.device)
    plan.call("pty_intensities", ptr(O), ptr(P), ptr(I))
    Iref = np.fft.fftshift(np.abs(np.fft.fft2(orc.make_exits(rnd["O"], rnd["P"], rnd["R"]))) ** 2,
                           axes=(-2, -1))
    assert rel(I.cpu().numpy(), Iref) < 4e-6


def c4_small(seed=4, side=3, step=36):
    """An 8-ish frame problem shaped like the 512^2 workload (background, Poisson, beamstop)."""
    rng = np.random.default_rng(seed)
    U = N + step * (side - 1) + 8
    O = (0.5 + 0.5 * smooth01(rng, (U, U))) * np.exp(1j * np.pi * (smooth01(rng, (U, U)) - 0.5))
    y, x = np.mgrid[:N, :N] - N / 2
    r = np.sqrt(x ** 2 + y ** 2)
    P = np.exp(-np.clip(r - 128, 0, None) ** 2 / 128.0) * (r < 176) * np.exp(1j * 0.0001 * r ** 2)
    pos = np.arange(side) * step + 4
    R = -np.stack(np.meshgrid(pos, pos, indexing="ij"), -1).reshape(-1, 2)
    R = np.clip(R + rng.integers(-4, 5, R.shape), -(U - N), 0)
    I = np.abs(np.fft.fft2(orc.make_exits(O, P, R))) ** 2
    blob = np.exp(-((x ** 2 + y ** 2) / (2 * 80.0 ** 2)))
    I = I + 0.01 * I.mean() * np.fft.ifftshift(blob)
    I = np.fft.fftshift(rng.poisson(I * (1e8 / I.sum(axis=(1, 2), keepdims=True))), axes=(-2, -1))
    M = np.ones((N, N), bool)
    M[r < 12] = False
    M[rng.random((N, N)) < 0.005] = False
    return I.astype(np.float32), R, P, O, M


def test_era_and_dm_m6_one_step_512():
    I, R, P, O, M = c4_small()
    np.random.seed(9)
    O_k, P_k, info = orc.ERA(I, R.copy(), P * np.exp(0.1j), None, 1, mask=M, method=6, dtype="double")
    b = info["background"]
    O_o, P_o, io = orc.ERA(I, R.copy(), P_k, O_k, 1, mask=M, method=6, background=b, dtype="double")
    O_g, P_g, ig = pty.ERA(I, R.copy(), P_k, O_k, 1, mask=M, method=6, background=b, dtype="double")
    assert rel(O_g, O_o) < 1e-5 and rel(P_g, P_o) < 1e-5
    assert ig["eMod"][0] == pytest.approx(io["eMod"][0], rel=1e-5)
    O_o, P_o, io = orc.DM(I, R.copy(), P_k, O_k, 1, mask=M, method=6, background=b, dtype="double")
    O_g, P_g, ig = pty.DM(I, R.copy(), P_k, O_k, 1, mask=M, method=6, background=b, dtype="double")
    assert rel(O_g, O_o) < 1e-5 and rel(P_g, P_o) < 1e-5
    assert ig["eMod"][0] == pytest.approx(io["eMod"][0], rel=1e-5)
