"""forward_sim's default object (forward_models.py:140-144: amplitude from the
'brog' test image scaled to [0, 1], phase from 'twain' scaled to [-pi, pi],
both resampled to shape_O by bagOfns.interpolate) against the objects the
reference itself recorded in tests/golden/forward_sim*.npz.

The two images ship with the reference, not with this package: the test reads
them from the reference checkout named by PTY_REFERENCE_ROOT, or from a
checkout next to this repository, and is skipped where neither exists.  Host
code only (no GPU): default_object is the host half of forward_sim.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def image_dir():
    roots = [os.environ.get("PTY_REFERENCE_ROOT"), os.path.join(os.path.dirname(HERE), "..", "reference")]
    for r in roots:
        if r and os.path.exists(os.path.join(r, "ptychography", "brog_256x256_32bit_big.raw")):
            return os.path.join(r, "ptychography")
    return None


@pytest.mark.skipif(image_dir() is None, reason="the reference's test images are not available here")
@pytest.mark.parametrize("fixture,shape", [("forward_sim.npz", (56, 56)), ("forward_sim_rect.npz", (80, 96))])
def test_default_object_matches_reference_fixture(fixture, shape, monkeypatch):
    monkeypatch.setenv("PTY_TEST_IMAGE_DIR", image_dir())
    from ptychography_gb300.forward_models import default_object
    O = default_object(shape)
    d = np.load(os.path.join(HERE, "golden", fixture))
    assert O.shape == d["O"].shape
    np.testing.assert_allclose(O, d["O"], rtol=0, atol=1e-13)
