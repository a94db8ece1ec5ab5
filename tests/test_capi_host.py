"""CPU-side checks of the C-ABI library and the Python host layer (no GPU calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

from ptychography_gb300 import _engine, _native
from oracle import ptycho_oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ptycho_gb300.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(pty_\w+)\s*\(", src, flags=re.M)))


def test_header_is_plain_c(tmp_path):
    """The boundary header needs no C++ and no CUDA headers: a C99 translation
    unit that includes it compiles with warnings as errors (what a cgo or
    JNI binding would compile)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "use_header.c"
    src.write_text('#include "ptycho_gb300.h"\nint main(void) { return pty_version() == 0; }\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.dirname(HEADER), "-c",
                        str(src), "-o", str(tmp_path / "use_header.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_header_declares_entry_points():
    names = header_functions()
    for must in ("pty_plan_create", "pty_era", "pty_dm", "pty_pmod_1", "pty_psup_O", "pty_psup_P"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = _native.load()
    for name in header_functions():
        assert hasattr(lib, name), name
        assert isinstance(getattr(lib, name), ctypes._CFuncPtr)


def test_ctypes_table_matches_header():
    assert set(_native.SIGNATURES) == set(header_functions())


def test_struct_layouts_match_c():
    # pty_options: 3 x int32, pad, int64, 2 x int32, 2 x double = 48 bytes
    assert ctypes.sizeof(_native.Options) == 48
    assert ctypes.sizeof(_native.Buffers) == 12 * ctypes.sizeof(ctypes.c_void_p)
    assert ctypes.sizeof(_native.Geometry) == 20


def test_version_and_shapes_without_gpu():
    lib = _native.load()
    assert lib.pty_version() >= 100
    for n in (32, 64, 128, 192, 256, 512):
        assert lib.pty_shape_supported(n, n) == 1
    assert lib.pty_shape_supported(32, 64) == 1
    assert lib.pty_shape_supported(48, 48) == 0
    assert lib.pty_shape_supported(100, 128) == 0


def test_frame_tile_candidates_without_gpu():
    lib = _native.load()
    want = {32: [1], 64: [1], 128: [1, 2], 192: [2], 256: [8, 4, 108], 512: [264, 116, 16]}
    for n, tiles in want.items():
        buf = (ctypes.c_int32 * 4)()
        cnt = ctypes.c_int32(0)
        assert lib.pty_frame_tile_candidates(n, n, buf, 4, ctypes.byref(cnt)) == 0
        assert [buf[i] for i in range(cnt.value)] == tiles
    cnt = ctypes.c_int32(0)
    assert lib.pty_frame_tile_candidates(48, 48, None, 0, ctypes.byref(cnt)) != 0


def test_plan_create_rejects_bad_geometry():
    lib = _native.load()
    plan = ctypes.c_void_p()
    R = np.zeros((2, 2), dtype=np.int64)
    g = _native.Geometry(2, 48, 48, 64, 64)          # no kernel for 48 x 48
    rc = lib.pty_plan_create(ctypes.byref(g), R.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                             ctypes.byref(plan))
    assert rc == 2 and b"not supported" in lib.pty_last_error()
    g = _native.Geometry(2, 32, 32, 40, 40)
    R = np.array([[0, 0], [-20, 0]], dtype=np.int64)  # window rows 20..52 > 40
    rc = lib.pty_plan_create(ctypes.byref(g), R.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                             ctypes.byref(plan))
    assert rc == 3 and b"outside the object" in lib.pty_last_error()
    with pytest.raises(ValueError):
        _native.check(rc)


def test_method_choice_matches_reference():
    assert _engine.choose_method(None, None, np.ones(1), None) == 1
    assert _engine.choose_method(None, np.ones(1), None, None) == 2
    assert _engine.choose_method(None, None, None, None) == 3
    assert _engine.choose_method(None, None, None, 1.0) == 6
    with pytest.raises(ValueError):
        _engine.choose_method(7, None, None, None)


def test_pmod_probe_schedule():
    c = _engine.pmod_probe_count
    assert c(False, 10) == 0 and c(None, 10) == 0
    assert c(True, 10) == 1            # i < True  -> i == 0 only
    assert c(3, 10) == 3 and c(2.5, 10) == 3
    assert c(np.inf, 10) == 10


def test_preamble_matches_oracle_rng_and_R_shift():
    rng = np.random.default_rng(0)
    I = rng.random((5, 32, 32)) * 10
    R = -rng.integers(0, 10, (5, 2)) + 3
    M = rng.random((32, 32)) > 0.1
    R1, R2 = R.copy(), R.copy()
    np.random.seed(3)
    pre = _engine.Preamble(I, R1, None, None, 1, M, None, 6, "single")
    np.random.seed(3)
    st = orc.preamble(I, R2, None, None, 1, M, None, 6, "single")
    assert np.array_equal(R1, R2) and R1.max(axis=0).tolist() == [0, 0]
    assert np.array_equal(pre.P, st["P"]) and np.array_equal(pre.O, st["O"])
    assert np.array_equal(pre.background, st["background"])
    assert np.array_equal(pre.mask.astype(bool), st["mask"])
    assert pre.I_norm == pytest.approx(float(st["I_norm"]), rel=1e-6)
    np.testing.assert_allclose(pre.Pamp, st["Pamp"], rtol=1e-6)


def test_preamble_leaves_the_callers_arrays_alone():
    """The reference copies P and O (era.py:492-493) and shifts R in place
    (era.py:504-505).  The preamble shifts R in place as well, converts P and
    O only when their dtype differs (a matching array is used as it is: it
    is only read, to upload), and writes to none of the caller's arrays."""
    rng = np.random.default_rng(1)
    I = (rng.random((4, 32, 32)) * 10).astype(np.float32)
    R = -rng.integers(0, 6, (4, 2)) + 2
    P = (rng.random((32, 32)) + 1j * rng.random((32, 32))).astype(np.complex64)
    O = (rng.random((40, 40)) + 1j * rng.random((40, 40))).astype(np.complex64)
    I0, P0, O0, R0 = I.copy(), P.copy(), O.copy(), R.copy()
    pre = _engine.Preamble(I, R, P, O, 1, 1, None, 3, "single")
    assert pre.P is P and pre.O is O                     # complex64 already: not copied
    assert np.array_equal(R, R0 - R0.max(axis=0))        # shifted in place, as the reference does
    assert np.array_equal(I, I0) and np.array_equal(P, P0) and np.array_equal(O, O0)
    pre64 = _engine.Preamble(I, R.copy(), P, O, 1, 1, None, 3, "double")
    assert pre64.P.dtype == np.complex128 and pre64.P is not P
    assert np.array_equal(pre64.P, P0.astype(np.complex128))
    assert np.array_equal(P, P0) and np.array_equal(O, O0)


def test_engine_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    I = np.ones((2, 32, 32))
    R = np.zeros((2, 2), dtype=int)
    with pytest.raises(RuntimeError, match="CUDA GPU"):
        _engine.run("era", I, R, np.ones((32, 32)), None, 1, 1, 1, None, 1, False, False, 1e-10,
                    None, True)


def test_preamble_rejects_malformed_inputs():
    """Inputs the reference would fail on with broadcast / unbound-name errors
    raise ValueError here (before any device work)."""
    I = np.ones((3, 32, 32))
    R = np.zeros((3, 2), dtype=np.int64)
    P = np.ones((32, 32))
    args = dict(OP_iters=1, mask=1, background=None, method=1, dtype=None)

    def pre(**kw):
        a = dict(I=I, R=R.copy(), P=P, O=None, **args)
        a.update(kw)
        return _engine.Preamble(a["I"], a["R"], a["P"], a["O"], a["OP_iters"], a["mask"],
                                a["background"], a["method"], a["dtype"])

    pre()                                                # well formed
    with pytest.raises(ValueError):
        pre(I=np.ones((32, 32)))                         # not a frame stack
    with pytest.raises(ValueError):
        pre(R=np.zeros((2, 2), dtype=np.int64))          # one offset per frame
    with pytest.raises(ValueError):
        pre(P=np.ones((16, 32)))                         # probe of another shape
    with pytest.raises(ValueError):
        pre(mask=np.ones((16, 16)))                      # mask of another shape
    with pytest.raises(ValueError):
        pre(dtype="half")
    with pytest.raises(ValueError):
        pre(method=0)
