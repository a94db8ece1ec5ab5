"""CXI files (display.py:21-117): without h5py both calls raise ImportError
naming it; with h5py a write / read round trip returns every array."""
import importlib.util

import numpy as np
import pytest

from ptychography_gb300 import cxi

HAVE_H5PY = importlib.util.find_spec("h5py") is not None


@pytest.mark.skipif(HAVE_H5PY, reason="h5py is installed")
def test_without_h5py_raises_import_error(tmp_path):
    with pytest.raises(ImportError, match="h5py"):
        cxi.write_cxi(np.zeros((1, 4, 4)), np.zeros((1, 4, 4)), None, None, None, None, None,
                      None, None, None, np.ones((4, 4)), None, fnam=str(tmp_path / "a.cxi"))
    with pytest.raises(ImportError, match="h5py"):
        cxi.read_cxi(str(tmp_path / "a.cxi"))


@pytest.mark.skipif(not HAVE_H5PY, reason="h5py is not installed")
def test_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    I = rng.random((3, 8, 8))
    P = rng.random((8, 8)) + 1j
    O = rng.random((12, 12)) + 0j
    R = -rng.integers(0, 4, (3, 2))
    M = rng.random((8, 8)) > 0.5
    e = [0.3, 0.2]
    fn = str(tmp_path / "r.cxi")
    cxi.write_cxi(I, I * 2, P, P * 2, O, O * 2, R, R, None, None, M, e, fnam=fn)
    out = cxi.read_cxi(fn, maxlen=2)
    np.testing.assert_array_equal(out[0], I[:2])
    np.testing.assert_array_equal(out[1], 2 * I[:2])
    np.testing.assert_array_equal(out[3], P * 2)
    assert out[8] is None and out[9] is None
    np.testing.assert_array_equal(out[10], M)
    np.testing.assert_array_equal(out[11], e)


def test_missing_directory_rejected(tmp_path):
    with pytest.raises((ValueError, ImportError)):
        cxi.write_cxi(np.zeros((1, 4, 4)), np.zeros((1, 4, 4)), None, None, None, None, None,
                      None, None, None, np.ones((4, 4)), None,
                      fnam=str(tmp_path / "no_such_dir" / "a.cxi"))
