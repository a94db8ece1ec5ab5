"""Size-independent properties at the full benchmark sizes, where the oracle
would take too long: 1024 frames of 256 x 256 over a 1024^2 object and 4096
frames of 512 x 512 over a 2816^2 object (raster scans as the benchmark's).

* The modulus projections are idempotent: Pmod(Pmod(psi)) = Pmod(psi)
  (era.py:560-595; alpha = 1e-10 and FP32 rounding leave ~1e-6).
* The consistency projections reproduce the object / probe that formed the
  exit waves: psup_O(P O[R], P) = O wherever the heatmap is well above alpha,
  and psup_P(P O[R], O) = P (era.py:336-400).
* Parseval for the model intensities: sum_k I_i(k) = N^2 sum_x |P O_i|^2
  (the fftshift only reorders).
"""
import ctypes

import numpy as np
import pytest
import torch

from gpu_util import Plan, ptr, rel

pytestmark = pytest.mark.gpu

SIZES = {
    "256": dict(N=256, side=32, step=24),
    "512": dict(N=512, side=64, step=36),
}


@pytest.fixture(scope="module", params=list(SIZES))
def scan(request):
    c = SIZES[request.param]
    N, side, step = c["N"], c["side"], c["step"]
    rng = np.random.default_rng(N)
    pos = np.arange(side) * step + 4
    R = -np.stack(np.meshgrid(pos, pos, indexing="ij"), -1).reshape(-1, 2)
    R = R + rng.integers(-3, 4, R.shape)
    R = R - R.max(axis=0)
    U = N + int(R[:, 0].max() - R[:, 0].min())
    V = N + int(R[:, 1].max() - R[:, 1].min())
    n = len(R)
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(N)
    O = (0.5 + torch.rand((U, V), device=dev, generator=g)) * torch.exp(
        1j * torch.rand((U, V), device=dev, generator=g))
    y, x = np.mgrid[:N, :N] - N / 2
    r = np.sqrt(x ** 2 + y ** 2)
    P = torch.from_numpy((np.exp(-np.clip(r - N / 4, 0, None) ** 2 / 32.0) * (r < N / 3)
                          * np.exp(1j * 0.0005 * r ** 2)).astype(np.complex64)).to(dev)
    plan = Plan(n, N, N, U, V, R)
    yield dict(N=N, n=n, U=U, V=V, O=O.to(torch.complex64), P=P, plan=plan, gen=g, dev=dev)
    plan.close()


def test_modulus_projections_are_idempotent(scan):
    n, N, plan, dev, g = scan["n"], scan["N"], scan["plan"], scan["dev"], scan["gen"]
    psi = torch.randn((n, N, N), dtype=torch.complex64, device=dev, generator=g)
    amp = torch.rand((n, N, N), device=dev, generator=g) * 10
    plan.call("pty_pmod_1", ptr(amp), ptr(psi), None, 1e-10, None)
    once = psi.clone()
    plan.call("pty_pmod_1", ptr(amp), ptr(psi), None, 1e-10, None)
    assert (torch.linalg.vector_norm(psi - once) / torch.linalg.vector_norm(once)).item() < 5e-6
    del psi, once
    psi = torch.randn((n, N, N), dtype=torch.complex64, device=dev, generator=g)
    bg = torch.rand((n, N, N), device=dev, generator=g)
    plan.call("pty_pmod_7", ptr(amp), ptr(bg), ptr(psi), None, 1e-10, None)
    once, bg1 = psi.clone(), bg.clone()
    plan.call("pty_pmod_7", ptr(amp), ptr(bg), ptr(psi), None, 1e-10, None)
    assert (torch.linalg.vector_norm(psi - once) / torch.linalg.vector_norm(once)).item() < 5e-6
    assert (torch.linalg.vector_norm(bg - bg1) / torch.linalg.vector_norm(bg1)).item() < 5e-6


def test_consistency_projections_reproduce_object_and_probe(scan):
    n, N, U, V = scan["n"], scan["N"], scan["U"], scan["V"]
    plan, dev, O, P = scan["plan"], scan["dev"], scan["O"], scan["P"]
    psi = torch.empty((n, N, N), dtype=torch.complex64, device=dev)
    plan.call("pty_make_exits", ptr(O), ptr(P), ptr(psi))
    heat = torch.zeros((U, V), dtype=torch.float64, device=dev)
    O2 = torch.empty_like(O)
    plan.call("pty_psup_O", ptr(psi), ptr(P), ptr(heat), 1, ctypes.c_double(1e-10), ptr(O2))
    lit = heat > 1e-3 * heat.max()
    assert (torch.linalg.vector_norm((O2 - O)[lit]) / torch.linalg.vector_norm(O[lit])).item() < 1e-5
    heatO = torch.zeros((N, N), dtype=torch.float64, device=dev)
    P2 = torch.empty_like(P)
    plan.call("pty_psup_P", ptr(psi), ptr(O), ptr(heatO), 1, ctypes.c_double(1e-10), ptr(P2))
    assert rel(P2.cpu().numpy(), P.cpu().numpy()) < 1e-5


def test_intensities_satisfy_parseval(scan):
    n, N, plan, dev, O, P = scan["n"], scan["N"], scan["plan"], scan["dev"], scan["O"], scan["P"]
    I = torch.empty((n, N, N), dtype=torch.float32, device=dev)
    plan.call("pty_intensities", ptr(O), ptr(P), ptr(I))
    psi = torch.empty((n, N, N), dtype=torch.complex64, device=dev)
    plan.call("pty_make_exits", ptr(O), ptr(P), ptr(psi))
    lhs = I.double().sum(dim=(1, 2))
    rhs = (psi.abs().double() ** 2).sum(dim=(1, 2)) * (N * N)
    assert (torch.abs(lhs - rhs) / rhs).max().item() < 1e-5
