"""256x256 frames: the cluster frame kernels (the autotuned tile) against the oracle.

Operators are compared on random data (FP32 rounding of a 256^2 FFT round
trip: 3e-6 relative); ERA / DM one-step errors on a small 256^2 problem with
background, noise and a beamstop mask must stay within 1e-5 relative.
"""
import numpy as np
import pytest
import torch

import ptychography_gb300 as pty
from gpu_util import Plan, ptr, rel, to_dev
from oracle import ptycho_oracle as orc
from test_gpu_parity_c0 import smooth01

pytestmark = pytest.mark.gpu
N = 256


@pytest.fixture(scope="module")
def rnd():
    rng = np.random.default_rng(256)
    n, U, V = 3, 320, 336
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


def test_pmod_1_256(rnd, plan):
    psi = to_dev(rnd["ex"], np.complex64)
    amp, mask = to_dev(rnd["amp"], np.float32), to_dev(rnd["mask"], np.uint8)
    e = torch.zeros(1, dtype=torch.float64, device=psi.device)
    plan.call("pty_pmod_1", ptr(amp), ptr(psi), ptr(mask), 1e-10, ptr(e))
    ref, em = orc.pmod_1(rnd["amp"], rnd["ex"].copy(), rnd["mask"], 1e-10, True)
    assert rel(psi.cpu().numpy(), ref) < 3e-6
    assert float(e.cpu()[0]) == pytest.approx(em, rel=1e-5)


def test_pmod_7_256(rnd, plan):
    psi = to_dev(rnd["ex"], np.complex64)
    amp, mask = to_dev(rnd["amp"], np.float32), to_dev(rnd["mask"], np.uint8)
    bg = to_dev(rnd["bg"], np.float32)
    e = torch.zeros(1, dtype=torch.float64, device=psi.device)
    plan.call("pty_pmod_7", ptr(amp), ptr(bg), ptr(psi), ptr(mask), 1e-10, ptr(e))
    ref, bref, em = orc.pmod_7(rnd["amp"], rnd["bg"].copy(), rnd["ex"].copy(), rnd["mask"], 1e-10, True)
    assert rel(psi.cpu().numpy(), ref) < 3e-6
    # b * f weights the small-|F| pixels, whose FP32 relative error is largest
    assert rel(bg.cpu().numpy(), bref) < 1e-5
    assert float(e.cpu()[0]) == pytest.approx(em, rel=1e-5)


def test_intensities_and_model_error_256(rnd, plan):
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


def c1_small(seed=1, side=4, step=24, U=None):
    """A 16-frame problem shaped like the 256^2 workload: background, Poisson, beamstop."""
    rng = np.random.default_rng(seed)
    U = U or N + step * (side - 1) + 8
    O = (0.5 + 0.5 * smooth01(rng, (U, U))) * np.exp(1j * np.pi * (smooth01(rng, (U, U)) - 0.5))
    y, x = np.mgrid[:N, :N] - N / 2
    r = np.sqrt(x ** 2 + y ** 2)
    P = np.exp(-np.clip(r - 64, 0, None) ** 2 / 32.0) * (r < 88) * np.exp(1j * 0.0005 * r ** 2)
    pos = np.arange(side) * step + 4
    R = -np.stack(np.meshgrid(pos, pos, indexing="ij"), -1).reshape(-1, 2)
    R = np.clip(R + rng.integers(-3, 4, R.shape), -(U - N), 0)
    ex = orc.make_exits(O, P, R)
    I = np.abs(np.fft.fft2(ex)) ** 2
    blob = np.exp(-((x ** 2 + y ** 2) / (2 * 40.0 ** 2)))
    I = I + 0.01 * I.mean() * np.fft.ifftshift(blob)
    I = np.fft.fftshift(rng.poisson(I * (1e6 / I.sum(axis=(1, 2), keepdims=True))), axes=(-2, -1))
    M = np.ones((N, N), bool)
    M[r < 12] = False
    M[rng.random((N, N)) < 0.005] = False
    return I.astype(np.float32), R, P, O, M


@pytest.fixture(scope="module")
def c1s():
    return c1_small()


def test_era_m6_one_step_256(c1s):
    I, R, P, O, M = c1s
    np.random.seed(7)
    O_k, P_k, info = orc.ERA(I, R.copy(), P * np.exp(0.1j), None, 2, mask=M, method=6, dtype="double")
    b = info["background"]            # fftshift(b)^2 == the background input convention
    O_o, P_o, io = orc.ERA(I, R.copy(), P_k, O_k, 1, mask=M, method=6, background=b, dtype="double")
    O_g, P_g, ig = pty.ERA(I, R.copy(), P_k, O_k, 1, mask=M, method=6, background=b, dtype="double")
    assert rel(O_g, O_o) < 1e-5 and rel(P_g, P_o) < 1e-5
    assert ig["eMod"][0] == pytest.approx(io["eMod"][0], rel=1e-5)
    assert rel(ig["background"], io["background"]) < 1e-5


def test_dm_m6_one_step_256(c1s):
    I, R, P, O, M = c1s
    np.random.seed(8)
    O_k, P_k, info = orc.ERA(I, R.copy(), P * np.exp(0.1j), None, 2, mask=M, method=6, dtype="double")
    b = info["background"]
    O_o, P_o, io = orc.DM(I, R.copy(), P_k, O_k, 1, mask=M, method=6, background=b, dtype="double")
    O_g, P_g, ig = pty.DM(I, R.copy(), P_k, O_k, 1, mask=M, method=6, background=b, dtype="double")
    assert rel(O_g, O_o) < 1e-5 and rel(P_g, P_o) < 1e-5
    assert ig["eMod"][0] == pytest.approx(io["eMod"][0], rel=1e-5)


@pytest.mark.parametrize("kind,method", [("era", 1), ("era", 3), ("dm", 1), ("dm", 3)])
def test_plain_methods_one_step_256(c1s, kind, method):
    """The EXIT1 / DM1 frame ops and the object / probe gathers at 256^2: one
    iteration from the oracle's FP64 state within 1e-5 relative."""
    I, R, P, O, M = c1s
    np.random.seed(9)
    O_k, P_k, _ = orc.ERA(I, R.copy(), P * np.exp(0.1j), None, 2, mask=M, method=3, dtype="double")
    fo, fg = (orc.ERA, pty.ERA) if kind == "era" else (orc.DM, pty.DM)
    P_in = P_k if method == 3 else P
    res_o = fo(I, R.copy(), P_in, O_k, 1, mask=M, method=method, dtype="double")
    res_g = fg(I, R.copy(), P_in, O_k, 1, mask=M, method=method, dtype="double")
    assert rel(res_g[0], res_o[0]) < 1e-5
    if method == 3:
        assert rel(res_g[1], res_o[1]) < 1e-5
    assert res_g[-1]["eMod"][0] == pytest.approx(res_o[-1]["eMod"][0], rel=1e-5)
