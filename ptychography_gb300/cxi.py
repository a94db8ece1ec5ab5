"""CXI-style result files: ``write_cxi`` / ``read_cxi`` (ptychography/display.py:21-117).

The same layout as the reference: an HDF5 file with groups ``input`` and
``output``; ``input`` holds ``I`` (gzip-compressed when ``compress``), ``M`` and,
when given, ``P``, ``O``, ``R``, ``B``; ``output`` holds ``I`` and, when given,
``P``, ``O``, ``R``, ``B``, ``eMod``.  ``write_cxi`` replaces an existing file
and rejects a missing or non-directory parent path with ValueError, as the
reference does.  ``read_cxi`` returns the same 12-tuple, the intensity stacks
cut to their first ``maxlen`` frames, and closes the file, also an open h5py
file it was given, as the reference does (the reference's read of a file
name refers to an unbound name before opening it; a file name works here).

HDF5 access needs h5py, which is imported when a file is written or read; on
a machine without it both functions raise ImportError.  The reconstruction
engine does not depend on this module.
"""
import os

_KEYS = ("P", "O", "R", "B")


def _h5py():
    try:
        import h5py
    except ImportError as e:  # pragma: no cover - depends on the machine
        raise ImportError("CXI files need h5py, which is not installed") from e
    return h5py


def _replace_target(fnam):
    out_dir = os.path.split(os.path.realpath(fnam))[0]
    if not os.path.exists(out_dir):
        raise ValueError("specified path does not exist: %s" % out_dir)
    if not os.path.isdir(out_dir):
        raise ValueError("specified path is not a directory: %s" % out_dir)
    if os.path.exists(fnam):
        os.remove(fnam)


def write_cxi(I_in, I_out, P_in, P_out, O_in, O_out, R_in, R_out, B_in, B_out, M, eMod,
              fnam="output.cxi", compress=True):
    """Write inputs and results to ``fnam`` (display.py:21-58); overwrites it."""
    h5py = _h5py()
    _replace_target(fnam)
    gz = dict(compression="gzip") if compress else {}
    with h5py.File(fnam, "w") as f:
        gin = f.create_group("input")
        gin.create_dataset("I", data=I_in, **gz)
        gin.create_dataset("M", data=M)
        for k, v in zip(_KEYS, (P_in, O_in, R_in, B_in)):
            if v is not None:
                gin.create_dataset(k, data=v)
        gout = f.create_group("output")
        gout.create_dataset("I", data=I_out, **gz)
        for k, v in zip(_KEYS + ("eMod",), (P_out, O_out, R_out, B_out, eMod)):
            if v is not None:
                gout.create_dataset(k, data=v)


def read_cxi(fnam="output.cxi", maxlen=100):
    """Read a file written by ``write_cxi`` (display.py:61-117): returns
    (I_in, I_out, P_in, P_out, O_in, O_out, R_in, R_out, B_in, B_out, M, eMod)."""
    own = isinstance(fnam, (str, os.PathLike))
    f = _h5py().File(fnam, "r") if own else fnam
    try:
        gin, gout = f["input"], f["output"]
        get = lambda g, k: g[k][()] if k in g else None  # noqa: E731
        I_in = gin["I"][:maxlen]
        I_out = gout["I"][:maxlen]
        P_in, O_in, R_in, B_in = (get(gin, k) for k in _KEYS)
        P_out, O_out, R_out, B_out = (get(gout, k) for k in _KEYS)
        return (I_in, I_out, P_in, P_out, O_in, O_out, R_in, R_out, B_in, B_out, gin["M"][()],
                get(gout, "eMod"))
    finally:
        f.close()             # display.py:116 closes the file, also one it was given
