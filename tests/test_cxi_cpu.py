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


class _FakeH5:
    """An in-memory stand-in for the part of h5py that write_cxi / read_cxi
    use: File (by name), groups, create_dataset (recording its options),
    dataset slicing and [()]."""

    files = {}

    class Dataset:
        def __init__(self, data, opts):
            self.data, self.opts = np.array(data), dict(opts)

        def __getitem__(self, k):
            return self.data[()] if k == () else self.data[k]

    class Group(dict):
        def create_group(self, name):
            g = _FakeH5.Group()
            self[name] = g
            return g

        def create_dataset(self, name, data=None, **opts):
            self[name] = _FakeH5.Dataset(data, opts)
            return self[name]

    class File(Group):
        def __init__(self, name, mode):
            super().__init__()
            self.name, self.mode, self.closed = name, mode, False
            if mode == "w":
                open(name, "wb").close()
                _FakeH5.files[name] = self
            else:
                self.update(_FakeH5.files[name])

        def close(self):
            self.closed = True

        def __enter__(self):
            return self

        def __exit__(self, *a):
            self.close()


@pytest.fixture
def fake_h5py(monkeypatch):
    import sys
    import types
    mod = types.ModuleType("h5py")
    mod.File = _FakeH5.File
    _FakeH5.files = {}
    monkeypatch.setitem(sys.modules, "h5py", mod)
    return _FakeH5


def test_layout_matches_display_py(tmp_path, fake_h5py):
    """The file layout of display.py:21-58: groups input / output; input holds
    I (gzip when compress), M and the given P, O, R, B; output holds I (gzip)
    and the given P, O, R, B, eMod; None entries are left out.  read_cxi
    (display.py:61-117) returns them, the stacks cut to maxlen frames."""
    rng = np.random.default_rng(1)
    I = rng.random((5, 4, 4))
    P, O = rng.random((4, 4)) + 1j, rng.random((6, 6)) + 0j
    R, M, B = -rng.integers(0, 3, (5, 2)), rng.random((4, 4)) > 0.3, rng.random((4, 4))
    fn = str(tmp_path / "x.cxi")
    cxi.write_cxi(I, 2 * I, P, None, O, 2 * O, R, None, B, None, M, [0.5, 0.25], fnam=fn)
    f = fake_h5py.files[fn]
    assert set(f) == {"input", "output"}
    assert set(f["input"]) == {"I", "M", "P", "O", "R", "B"}
    assert set(f["output"]) == {"I", "O", "eMod"}
    assert f["input"]["I"].opts == {"compression": "gzip"}
    assert f["output"]["I"].opts == {"compression": "gzip"}
    assert f["input"]["M"].opts == {} and f["output"]["eMod"].opts == {}
    out = cxi.read_cxi(fn, maxlen=3)
    np.testing.assert_array_equal(out[0], I[:3])
    np.testing.assert_array_equal(out[1], 2 * I[:3])
    np.testing.assert_array_equal(out[2], P)
    assert out[3] is None and out[7] is None and out[9] is None
    np.testing.assert_array_equal(out[5], 2 * O)
    np.testing.assert_array_equal(out[6], R)
    np.testing.assert_array_equal(out[8], B)
    np.testing.assert_array_equal(out[10], M)
    np.testing.assert_array_equal(out[11], [0.5, 0.25])
    # uncompressed, and an existing file is replaced
    cxi.write_cxi(I, I, None, None, None, None, None, None, None, None, M, None, fnam=fn, compress=False)
    f = fake_h5py.files[fn]
    assert f["input"]["I"].opts == {} and set(f["output"]) == {"I"}
    # an open file is read and closed, as display.py:116 does
    g = fake_h5py.File(fn, "r")
    cxi.read_cxi(g)
    assert g.closed
