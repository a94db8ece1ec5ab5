"""pty_amp_and_norm: the amplitudes equal pty_amp_from_intensity's and I_norm
equals sum(mask * I) (era.py:495) to double rounding."""

import numpy as np
import pytest
import torch

from gpu_util import Plan, ptr, to_dev
from ptychography_gb300 import _native

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("N,use_mask", [(64, True), (256, False), (128, True)])
def test_amp_and_norm(dtype, N, use_mask):
    rng = np.random.default_rng(N)
    n, U = 6, N + 20
    R = -rng.integers(0, U - N + 1, (n, 2))
    I = (rng.random((n, N, N)) * 1000).astype(dtype)
    mask = rng.random((N, N)) > 0.1
    plan = Plan(n, N, N, U, U, R)
    try:
        I_d = to_dev(I)
        mask_d = to_dev(np.fft.ifftshift(mask).astype(np.uint8)) if use_mask else None
        a1 = torch.empty((n, N, N), dtype=torch.float32, device=I_d.device)
        a2 = torch.empty_like(a1)
        norm = torch.zeros(1, dtype=torch.float64, device=I_d.device)
        plan.call("pty_amp_from_intensity", ptr(I_d), int(dtype == np.float64), ptr(a1))
        plan.call("pty_amp_and_norm", ptr(I_d), int(dtype == np.float64), ptr(mask_d), ptr(a2),
                  ptr(norm))
    finally:
        plan.close()
    np.testing.assert_array_equal(a1.cpu().numpy(), a2.cpu().numpy())
    want = np.sum((mask if use_mask else 1.0) * I.astype(np.float64))
    assert float(norm.cpu()[0]) == pytest.approx(want, rel=1e-12)
    # the same amplitudes as the reference's preamble: ifftshift(sqrt(I))
    ref = np.fft.ifftshift(np.sqrt(I.astype(np.float64)), axes=(-2, -1)).astype(np.float32)
    np.testing.assert_allclose(a2.cpu().numpy(), ref, rtol=1e-6)
