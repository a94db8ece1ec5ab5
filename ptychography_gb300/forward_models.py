"""Drop-in ``forward_sim`` (ptychography/forward_models.py:12-203).

The probe, scan grid, random offsets, background, mask and Poisson statistics
follow the reference step by step, drawing from NumPy's global RNG in the same
order.  The diffraction intensities ``|FFT(P * O[R])|^2`` of all frames are
computed on the GPU by the library's fused frame kernel.

The reference builds the object from two test images shipped beside its
source.  When the directory holding them is given by ``PTY_TEST_IMAGE_DIR``
the same object is built from them; otherwise a smooth random object of the
requested shape is used (amplitude in [0, 1], phase in [-pi, pi]) from a
private RNG, so the global RNG stream is the reference's either way.  An object
can also be passed explicitly with ``O=``.
"""
import ctypes
import os

import numpy as np

from . import _native


def _probe(shape, A, defocus, photons_pupil):
    """forward_models.py:124-138."""
    f0 = np.fft.fftfreq(shape[0], 1 / float(shape[0]))
    f1 = np.fft.fftfreq(shape[1], 1 / float(shape[1]))
    i, j = np.meshgrid(f0, f1, indexing="ij")
    q2 = np.fft.fftshift(i ** 2 + j ** 2)
    P = (q2 < A ** 2).astype(np.complex128) * np.sqrt(photons_pupil)
    P *= np.exp(-1.0J * np.pi * defocus * q2)
    return np.fft.fftshift(np.fft.ifftn(np.fft.ifftshift(P)))


def _scale(a, lo, hi):
    return (a - a.min()) / (a.max() - a.min()) * (hi - lo) + lo


def _image(name, shape):
    import scipy.ndimage as ndi
    path = os.path.join(os.environ["PTY_TEST_IMAGE_DIR"], "%s_256x256_32bit_big.raw" % name)
    a = np.fromfile(path, dtype=">f4").reshape(256, 256).astype(np.float32)
    if tuple(shape) != (256, 256):
        coeffs = ndi.spline_filter(a)
        coords = np.mgrid[0:255:1j * shape[0], 0:255:1j * shape[1]]
        a = ndi.map_coordinates(coeffs, coords, prefilter=False)
    return a


def default_object(shape_O):
    """The reference's test object, or a smooth random stand-in (see module doc)."""
    if os.environ.get("PTY_TEST_IMAGE_DIR"):
        amp = _scale(_image("brog", shape_O), 0.0, 1.0)
        phase = _scale(_image("twain", shape_O), -np.pi, np.pi)
        return amp * np.exp(1J * phase)
    import scipy.ndimage as ndi
    rs = np.random.RandomState(20150601)
    a = ndi.gaussian_filter(rs.random_sample(shape_O), 4.0)
    p = ndi.gaussian_filter(rs.random_sample(shape_O), 4.0)
    return _scale(a, 0.0, 1.0) * np.exp(1J * _scale(p, -np.pi, np.pi))


def diffraction_intensities(O, P, R):
    """ifftshift(|FFT2(P * O[R_i])|^2) for every scan position, on the GPU (float64 out)."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("ptychography_gb300 runs on a CUDA GPU; none is available")
    lib = _native.load()
    n = len(R)
    N0, N1 = P.shape
    U, V = O.shape
    dev = torch.device("cuda", torch.cuda.current_device())
    geom = _native.Geometry(n, N0, N1, U, V)
    R64 = np.ascontiguousarray(R[:, :2], dtype=np.int64)
    plan = ctypes.c_void_p()
    _native.check(lib.pty_plan_create(ctypes.byref(geom),
                                      R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                      ctypes.byref(plan)))
    try:
        O_d = torch.from_numpy(np.ascontiguousarray(O.astype(np.complex64))).to(dev)
        P_d = torch.from_numpy(np.ascontiguousarray(P.astype(np.complex64))).to(dev)
        I_d = torch.empty((n, N0, N1), dtype=torch.float32, device=dev)
        stream = torch.cuda.current_stream(dev)
        _native.check(lib.pty_intensities(plan, ctypes.c_void_p(O_d.data_ptr()),
                                          ctypes.c_void_p(P_d.data_ptr()),
                                          ctypes.c_void_p(I_d.data_ptr()),
                                          ctypes.c_void_p(stream.cuda_stream)))
        stream.synchronize()
        # the kernel writes fftshift(|F|^2); the reference's ifftshift is the same
        # permutation for the even frame sizes the kernels support
        return I_d.cpu().numpy().astype(np.float64)
    finally:
        lib.pty_plan_destroy(plan)


def forward_sim(shape_P=(32, 64), shape_O=(128, 128), A=14, defocus=0., photons_pupil=1,
                ny=10, nx=10, random_offset=None, background=None, mask=None,
                counting_statistics=False, O=None):
    """Simulate a ptychographic data set; returns ``I, R, M, P, O, B`` (forward_models.py:12)."""
    shape = tuple(shape_P)
    P = _probe(shape, A, defocus, photons_pupil)
    if O is None:
        O = default_object(tuple(shape_O))
    O = np.asarray(O, dtype=np.complex128)
    shape_O = O.shape
    ys = np.rint(np.linspace(0, P.shape[0] - O.shape[0], ny)).astype(int)   # :149-152
    xs = np.rint(np.linspace(0, P.shape[1] - O.shape[1], nx)).astype(int)
    ys, xs = np.meshgrid(ys, xs, indexing="ij")
    R = np.stack([ys.ravel(), xs.ravel()], axis=1)
    if random_offset is not None:                                           # :155-160
        R += (np.random.random(R.shape) * int(random_offset)).astype(int)
        R[R > 0] = 0
        R[:, 0][R[:, 0] < shape[0] - shape_O[0]] = shape[0] - shape_O[0]
        R[:, 1][R[:, 1] < shape[1] - shape_O[1]] = shape[1] - shape_O[1]
    R[:, 0] -= R[:, 0].max()
    R[:, 1] -= R[:, 1].max()
    I = diffraction_intensities(O, P, R)                                   # :167-171
    if background is not None:                                              # :174-179
        B = np.rint(np.random.random(I[0].shape) * background)
        I += B
    else:
        B = 0
    if mask is not None:                                                    # :182-188
        ss = (np.random.random(mask) * I.shape[1]).astype(int)
        fs = (np.random.random(mask) * I.shape[2]).astype(int)
        M = np.ones(I[0].shape, dtype=bool)
        M[ss, fs] = False
    else:
        M = 1
    if counting_statistics:                                                 # :191-192
        I = np.random.poisson(lam=I)
    if not (isinstance(B, int) and B == 0):
        B = B.astype(I.dtype)
    return I, R, M, P, O, B
