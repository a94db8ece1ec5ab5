"""The MT19937 sequence form used by pty_legacy_random_background, checked on
the CPU against NumPy's own legacy global generator.

The device kernel computes x[m] = x[m-227] ^ twist(x[m-624], x[m-623]) for
m >= 624 from the state array x[0..623], outputs temper(x[pos + k]) and forms
doubles from output pairs; the state after drawing W words is the 624-word
block holding the last word, with position (pos + W - 1) % 624 + 1.  This
NumPy restatement of exactly that arithmetic must reproduce
np.random.random bit for bit, and the final state np.random.get_state().
"""
import numpy as np
import pytest


def seq_extend(key, total):
    x = np.zeros(total, dtype=np.uint64)
    x[:624] = key
    for m0 in range(624, total, 227):
        m = np.arange(m0, min(m0 + 227, total))
        lo, hi = x[m - 624], x[m - 623]
        y = (lo & 0x80000000) | (hi & 0x7fffffff)
        x[m] = x[m - 227] ^ (y >> 1) ^ np.where(y & 1, 0x9908b0df, 0).astype(np.uint64)
    return x


def temper(y):
    y = y ^ (y >> 11)
    y = y ^ ((y << 7) & 0x9d2c5680)
    y = y ^ ((y << 15) & 0xefc60000)
    y = y ^ (y >> 18)
    return y & 0xffffffff


def draw(key, pos, count):
    e = pos + 2 * count
    last_block = (e - 1) // 624
    x = seq_extend(key, (last_block + 1) * 624)
    w = temper(x[pos:e])
    a, b = w[0::2] >> 5, w[1::2] >> 6
    u = (a.astype(np.float64) * 67108864.0 + b.astype(np.float64)) / 9007199254740992.0
    return u, x[last_block * 624:(last_block + 1) * 624].astype(np.uint32), (e - 1) % 624 + 1


@pytest.mark.parametrize("seed,skip,count", [(0, 0, 1), (1, 0, 5000), (7, 3, 777), (11, 311, 312),
                                             (13, 623, 2000), (2, 1, 100000)])
def test_sequence_form_matches_numpy(seed, skip, count):
    np.random.seed(seed)
    np.random.random(skip)                  # move pos (each double takes two words)
    st = np.random.get_state()
    u, key2, pos2 = draw(st[1].astype(np.uint64), st[2], count)
    ref = np.random.random(count)
    np.testing.assert_array_equal(u, ref)
    st2 = np.random.get_state()
    assert pos2 == st2[2]
    np.testing.assert_array_equal(key2, st2[1])


def test_float32_path_matches_astype():
    """float32(u) + 0.1 in float32 equals the reference's astype(float32) + 0.1."""
    np.random.seed(3)
    u = np.random.random(10000)
    ref = u.astype(np.float32) + 0.1
    assert ref.dtype == np.float32
    v = np.round(u * 2.0 ** 53).astype(np.uint64)             # the 53-bit integer
    f = v.astype(np.float32) * np.float32(2.0 ** -53)
    np.testing.assert_array_equal(f + np.float32(0.1), ref)


@pytest.mark.parametrize("seed,blocks", [(3, 1), (8, 5), (21, 210), (40, 1025)])
def test_jump_ahead_matches_numpy(seed, blocks):
    """The library's jump-ahead (x^J mod phi applied to a window, the same
    polynomials the device draw uses to start its segments) lands on NumPy's
    own state after J = 624 * blocks raw words."""
    import ctypes
    from ptychography_gb300 import _native
    lib = _native.load()
    np.random.seed(seed)
    key0 = np.ascontiguousarray(np.random.get_state()[1], dtype=np.uint32)
    np.random.random(312 * blocks)                 # 624 * blocks words, whole blocks
    st = np.random.get_state()
    assert st[2] == 624
    want = np.asarray(st[1], dtype=np.uint32)
    got = np.empty(624, dtype=np.uint32)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    _native.check(lib.pty_legacy_random_jump(key0.ctypes.data_as(u32p), 624 * blocks,
                                             got.ctypes.data_as(u32p)))
    np.testing.assert_array_equal(got[1:], want[1:])
    assert got[0] >> 31 == want[0] >> 31            # only its top bit is state


def test_jump_rejects_bad_arguments():
    import ctypes
    from ptychography_gb300 import _native
    lib = _native.load()
    key = np.zeros(624, dtype=np.uint32)
    out = np.empty(624, dtype=np.uint32)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    assert lib.pty_legacy_random_jump(key.ctypes.data_as(u32p), -1, out.ctypes.data_as(u32p)) != 0
    assert lib.pty_legacy_random_jump(None, 5, out.ctypes.data_as(u32p)) != 0
