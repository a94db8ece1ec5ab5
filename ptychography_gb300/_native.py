"""ctypes binding of libptycho_gb300.so (declared in include/ptycho_gb300.h).

Loading fails loudly: there is no CPU path behind this module.  On a machine
without a GPU the library still loads (its symbols can be inspected), but the
entry points need a CUDA device.
"""
import ctypes
import os

from . import _build

_lib = None

c_int32, c_int64, c_double, c_void_p = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p


class Geometry(ctypes.Structure):
    _fields_ = [("n_frames", c_int32), ("N0", c_int32), ("N1", c_int32), ("U", c_int32), ("V", c_int32)]


class Buffers(ctypes.Structure):
    _fields_ = [("O", c_void_p), ("P", c_void_p), ("psi", c_void_p), ("amp", c_void_p),
                ("mask", c_void_p), ("background", c_void_p), ("Pamp", c_void_p),
                ("background_mean", c_void_p), ("heatmap", c_void_p), ("intensities", c_void_p),
                ("eMod", c_void_p), ("eCon", c_void_p)]


class Options(ctypes.Structure):
    _fields_ = [("method", c_int32), ("OP_iters0", c_int32), ("OP_iters1", c_int32),
                ("Pmod_probe", c_int64), ("probe_centering", c_int32), ("use_graph", c_int32),
                ("alpha", c_double), ("I_norm", c_double)]


# (name, argtypes); every function returns int status unless listed in _RESTYPES
SIGNATURES = {
    "pty_plan_create": [ctypes.POINTER(Geometry), ctypes.POINTER(c_int64), ctypes.POINTER(c_void_p)],
    "pty_plan_destroy": [c_void_p],
    "pty_plan_geometry": [c_void_p, ctypes.POINTER(Geometry)],
    "pty_era": [c_void_p, ctypes.POINTER(Buffers), ctypes.POINTER(Options), c_int32,
                ctypes.POINTER(c_int32), c_void_p],
    "pty_dm": [c_void_p, ctypes.POINTER(Buffers), ctypes.POINTER(Options), c_int32,
               ctypes.POINTER(c_int32), c_void_p],
    "pty_run_batch": [c_int32, ctypes.POINTER(c_void_p), ctypes.POINTER(Buffers), ctypes.POINTER(Options),
                      c_int32, c_int32, ctypes.POINTER(c_int32), c_void_p],
    "pty_make_exits": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "pty_pmod_1": [c_void_p, c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p],
    "pty_pmod_7": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p],
    "pty_Pmod_P": [c_void_p, c_void_p, c_void_p, c_void_p, c_double, c_void_p],
    "pty_psup_O": [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_double, c_void_p, c_void_p],
    "pty_psup_P": [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_double, c_void_p, c_void_p],
    "pty_make_P_heatmap": [c_void_p, c_void_p, c_void_p, c_void_p],
    "pty_make_O_heatmap": [c_void_p, c_void_p, c_void_p, c_void_p],
    "pty_model_error_1": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_void_p,
                          c_void_p],
    "pty_intensities": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "pty_background_mean": [c_void_p, c_void_p, c_void_p, c_void_p],
    "pty_back_project": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "pty_amp_and_norm": [c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p, c_void_p],
    "pty_amp_from_intensity": [c_void_p, c_void_p, c_int32, c_void_p, c_void_p],
    "pty_psup_P_noalloc": [ctypes.POINTER(Geometry), ctypes.POINTER(c_int64), c_void_p, c_void_p,
                           c_void_p, c_int32, c_double, c_void_p, c_void_p],
    "pty_legacy_random_background": [ctypes.POINTER(ctypes.c_uint32), c_int32, ctypes.c_int64,
                                     c_int32, c_void_p, c_void_p, ctypes.POINTER(ctypes.c_uint32),
                                     ctypes.POINTER(c_int32), c_void_p],
    "pty_legacy_random_background_async": [ctypes.POINTER(ctypes.c_uint32), c_int32, ctypes.c_int64,
                                     c_int32, c_void_p, c_void_p, ctypes.POINTER(ctypes.c_uint32),
                                     ctypes.POINTER(c_int32), c_void_p],
    "pty_legacy_random_scratch_words": [c_int32, ctypes.c_int64],
    "pty_legacy_random_jump": [ctypes.POINTER(ctypes.c_uint32), ctypes.c_int64,
                               ctypes.POINTER(ctypes.c_uint32)],
    "pty_ws_gemm": [c_int32, c_int32, c_int32, c_void_p, c_int64, c_int64, c_void_p, c_int64, c_int64,
                    c_void_p, c_int64, c_int64, c_int32, c_void_p, c_void_p],
    "pty_ws_im2col": [c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p],
    "pty_ws_col2im": [c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p],
    "pty_ws_pool2": [c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p],
    "pty_ws_pool2_bwd": [c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p],
    "pty_ws_up2": [c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p],
    "pty_ws_up2_bwd": [c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p],
    "pty_ws_bias_act": [c_int64, c_int32, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p,
                        c_void_p, c_void_p],
    "pty_ws_act_bwd_scratch": [c_int64, c_int32],
    "pty_ws_act_bwd": [c_int64, c_int32, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p,
                       c_void_p],
    "pty_ws_loss": [c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "pty_ws_adam": [c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, ctypes.c_float,
                    ctypes.c_float, ctypes.c_float, ctypes.c_float, c_int32, c_void_p],
    "pty_ws_to_bf16": [c_int64, c_void_p, c_void_p, c_void_p],
    "pty_ws_add": [c_int64, c_void_p, c_void_p, c_void_p, c_void_p],
    "pty_ws_flip_weights": [c_int32, c_int32, c_void_p, c_void_p, c_void_p],
    "pty_ws_prep_bp": [c_int32, c_int32, c_int32, c_void_p, c_void_p, c_int32, c_void_p, c_void_p],
    "pty_ws_targets": [c_int32, c_int64, c_void_p, c_void_p, c_int32, ctypes.c_float, c_void_p, c_void_p,
                       c_void_p],
    "pty_ws_exits": [c_int32, c_int64, c_void_p, c_void_p, c_int32, c_void_p, c_void_p],
    "pty_ws_conv3x3_tc": [c_int32, c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                          c_int32, c_void_p, c_void_p, c_void_p, c_void_p],
    "pty_ws_conv3x3_tc_f32": [c_int32, c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                              c_void_p],
    "pty_ws_shift_transpose": [c_int32, c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p],
    "pty_ws_wgrad_tc_scratch": [c_int32, c_int32, c_int32, c_int32, c_int32],
    "pty_ws_wgrad_tc": [c_int32, c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p,
                        c_int64, c_void_p],
    "pty_timeout_status": [ctypes.POINTER(c_int32)],
    "pty_ws_conv3x3_direct": [c_int32, c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                              c_int32, c_void_p, c_void_p, c_void_p, c_void_p],
    "pty_ws_crop_center": [c_int32, c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, ctypes.c_float,
                           c_void_p, c_void_p],
    "pty_ws_upsample_object": [c_int32, c_int32, c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p],
    "pty_ws_align_phase": [c_int32, c_int32, c_int32, c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                           c_void_p],
    "pty_shape_supported": [c_int32, c_int32],
    "pty_frame_tile_candidates": [c_int32, c_int32, ctypes.POINTER(c_int32), c_int32,
                                  ctypes.POINTER(c_int32)],
    "pty_get_frame_tile": [c_int32, c_int32, c_int32, ctypes.POINTER(c_int32)],
    "pty_set_frame_tile": [c_int32, c_int32, c_int32, c_int32],
    "pty_last_error": [],
    "pty_version": [],
    "pty_launch_count": [],
}
_RESTYPES = {"pty_last_error": ctypes.c_char_p, "pty_launch_count": ctypes.c_int64,
             "pty_legacy_random_scratch_words": ctypes.c_int64,
             "pty_ws_act_bwd_scratch": ctypes.c_int64, "pty_ws_wgrad_tc_scratch": ctypes.c_int64}


class PtyError(RuntimeError):
    """A non-zero status from the CUDA library."""

    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (building first if needed) and return the ctypes library handle."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libptycho_gb300.so is not built: run python -m ptychography_gb300._build")
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, ctypes.c_int)
    _lib = lib
    return lib


def check(rc):
    """Raise PtyError (ValueError subclasses for argument/range errors) on failure."""
    if rc == 0:
        return
    msg = load().pty_last_error().decode(errors="replace")
    if rc in (1, 2, 3):
        raise PtyValueError(rc, msg)
    raise PtyError(rc, msg)


class PtyValueError(PtyError, ValueError):
    """Bad argument, unsupported frame shape or scan window outside the object."""


def plan_geometry(plan_h):
    """The Geometry a plan handle was created with."""
    g = Geometry()
    check(load().pty_plan_geometry(plan_h, ctypes.byref(g)))
    return g
