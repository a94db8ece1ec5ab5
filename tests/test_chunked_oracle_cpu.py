"""The chunked FP64 oracle (torch float64 on the CPU here) against the NumPy
oracle, which the golden fixtures pin to the reference itself.

A small seeded problem (24 frames of 32 x 32 on a jittered raster, a random
object and probe, a beamstop mask and a smooth background) runs three ERA and
three DM iterations of each method (1-6) through both; every output must
agree to 1e-11 relative (float64 rounding of the transforms: the NumPy
oracle uses pocketfft, torch its own FFT), with the two exceptions the test
states (a settled eCon, DM method 5's background).  Frame chunks of 5 make
every chunk loop run ragged.
"""
import numpy as np
import pytest

from oracle import chunked_fp64 as ck
from oracle import ptycho_oracle as orc

torch = pytest.importorskip("torch")


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _problem(seed=3):
    rng = np.random.default_rng(seed)
    N, side, step = 32, 5, 9
    R = np.array([(-step * i - rng.integers(0, 3), -step * j - rng.integers(0, 3))
                  for i in range(side) for j in range(side)][:24], dtype=np.int64)
    U = N + int(R[:, 0].max() - R[:, 0].min())
    V = N + int(R[:, 1].max() - R[:, 1].min())
    O = (0.6 + 0.4 * rng.random((U, V))) * np.exp(1j * rng.uniform(-1, 1, (U, V)))
    y, x = np.mgrid[:N, :N] - N // 2
    P = (np.hypot(y, x) < 10).astype(float) * np.exp(1j * 0.01 * (x ** 2 + y ** 2))
    RR = R - R.max(axis=0)
    ex = orc.make_exits(O, P, RR)
    I = np.fft.fftshift(np.abs(np.fft.fftn(ex, axes=(-2, -1))) ** 2, axes=(-2, -1))
    B = 0.01 * I.mean() * np.exp(-(x ** 2 + y ** 2) / 60.0)
    I = I + B
    M = np.hypot(y, x) > 2
    P0 = P * np.exp(1j * 0.002 * (x ** 2 + y ** 2))
    O0 = np.ones((U, V), np.complex128)
    return I, R, P0, O0, M, B


@pytest.mark.parametrize("algo", ["ERA", "DM"])
@pytest.mark.parametrize("method", [1, 2, 3, 4, 5, 6])
def test_chunked_matches_numpy_oracle(algo, method):
    I, R, P0, O0, M, B = _problem()
    bg = B if method >= 4 else None
    fn = getattr(orc, algo)
    out = fn(I, R.copy(), P0.copy(), O0.copy(), 3, mask=M, background=bg, method=method, dtype="double")
    pb = ck.Problem(I, R, P0, O0, M, bg, torch.device("cpu"), chunk=5)
    O_c, P_c, info_c = getattr(ck, algo)(pb, 3, method)
    if method in (1, 4):
        O_o, info_o = out
        P_o = P0
    elif method in (2, 5):
        P_o, info_o = out
        O_o = O0
    else:
        O_o, P_o, info_o = out
    assert _rel(O_c.numpy(), O_o) < 1e-11
    assert _rel(P_c.numpy(), P_o) < 1e-11
    np.testing.assert_allclose(info_c["eMod"], info_o["eMod"], rtol=1e-11)
    # eCon relative to the first iteration's: a probe-only ERA run settles in
    # one step (eCon ~1e-11 after it), where only the absolute error means anything
    np.testing.assert_allclose(info_c["eCon"], info_o["eCon"], rtol=1e-9, atol=1e-12 * info_o["eCon"][0])
    if method >= 4:
        # DM method 5's background recursion amplifies the two FFT libraries'
        # last-bit differences: 1e-14, 3e-13, 9e-9 after 1, 2, 3 iterations
        tol = 1e-7 if (algo, method) == ("DM", 5) else 1e-11
        assert _rel(info_c["background"].numpy(), info_o["background"]) < tol


def test_unsupported_options_raise():
    I, R, P0, O0, M, B = _problem()
    pb = ck.Problem(I, R, P0, O0, M, None, torch.device("cpu"), chunk=5)
    with pytest.raises(NotImplementedError):
        ck.DM(pb, 1, 7)
    with pytest.raises(NotImplementedError):
        ck.ERA(pb, 1, 4)                        # a background method without the known background
    with pytest.raises(NotImplementedError):
        ck.DM(pb, 1, 5)


@pytest.mark.parametrize("algo", ["ERA", "DM"])
@pytest.mark.parametrize("method", [3, 6])
def test_chunked_centring_and_probe_modulus(algo, method):
    """Probe centring and the far-field probe constraint (Pmod_P for the first
    two iterations) against the NumPy oracle; the initial probe is off centre
    so that the centring rolls the probe, the object and (DM) the exit waves.

    Pmod_P sets |fftn P| to the initial probe's far-field modulus, so at
    frequencies where the current probe's transform is near zero it scales
    rounding noise of the two FFT libraries (pocketfft, torch) by a large
    factor: the two oracles then agree to 1e-6 (DM method 3 is the most
    sensitive), not 1e-11.  Without Pmod_P they agree to 1e-11 (above)."""
    I, R, P0, O0, M, B = _problem()
    P0 = np.roll(P0, (3, -2), axis=(0, 1))
    bg = B if method >= 4 else None
    fn = getattr(orc, algo)
    out = fn(I, R.copy(), P0.copy(), O0.copy(), 3, mask=M, background=bg, method=method, dtype="double",
             probe_centering=True, Pmod_probe=2)
    O_o, P_o, info_o = out
    pb = ck.Problem(I, R, P0, O0, M, bg, torch.device("cpu"), chunk=5)
    O_c, P_c, info_c = getattr(ck, algo)(pb, 3, method, probe_centering=True, Pmod_probe=2)
    # the object where the final probe lights it (heat > 1e-3 of its maximum):
    # after a roll, pixels the probe barely reaches divide rounding-level sums
    # by rounding-level heat, where the two FFT libraries' last bits differ
    heat = np.zeros(O_o.shape)
    RR = R - R.max(axis=0)
    for r0, r1 in RR:
        heat[-r0:-r0 + 32, -r1:-r1 + 32] += np.abs(P_o) ** 2
    lit = heat > 1e-3 * heat.max()
    assert _rel(O_c.numpy()[lit], O_o[lit]) < 1e-6
    assert _rel(P_c.numpy(), P_o) < 1e-6
    np.testing.assert_allclose(info_c["eMod"], info_o["eMod"], rtol=1e-6)
    np.testing.assert_allclose(info_c["eCon"], info_o["eCon"], rtol=1e-5)
    # the centring moved the probe back: its centre of mass is at the middle
    a = np.abs(P_c.numpy()) ** 2
    com = (np.arange(32) @ a.sum(axis=1) / a.sum(), np.arange(32) @ a.sum(axis=0) / a.sum())
    assert abs(com[0] - 16) <= 1.0 and abs(com[1] - 16) <= 1.0


@pytest.mark.parametrize("algo", ["ERA", "DM"])
@pytest.mark.parametrize("method", [3, 6])
@pytest.mark.parametrize("OP_iters", [(2, 1), (1, 3), (2, 3)])
def test_chunked_op_iters(algo, method, OP_iters):
    """OP_iters = (k, m): k object / probe rounds every m-th iteration and the
    object alone (with the cached, possibly stale heatmap) in between, five
    iterations so that both kinds run, against the NumPy oracle."""
    I, R, P0, O0, M, B = _problem()
    bg = B if method >= 4 else None
    fn = getattr(orc, algo)
    O_o, P_o, info_o = fn(I, R.copy(), P0.copy(), O0.copy(), 5, OP_iters=OP_iters, mask=M, background=bg,
                          method=method, dtype="double")
    pb = ck.Problem(I, R, P0, O0, M, bg, torch.device("cpu"), chunk=5)
    O_c, P_c, info_c = getattr(ck, algo)(pb, 5, method, OP_iters=OP_iters)
    assert _rel(O_c.numpy(), O_o) < 1e-11
    assert _rel(P_c.numpy(), P_o) < 1e-11
    np.testing.assert_allclose(info_c["eMod"], info_o["eMod"], rtol=1e-11)
    np.testing.assert_allclose(info_c["eCon"], info_o["eCon"], rtol=1e-9, atol=1e-12 * info_o["eCon"][0])
