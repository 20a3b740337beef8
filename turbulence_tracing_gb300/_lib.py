"""ctypes binding of libturbotrace.so (the C ABI declared in include/turbotrace.h).

The library is built in-tree by ``turbulence_tracing_gb300.build`` (nvcc,
sm_103a).  Loading never falls back to anything else: if the shared library
is missing or does not load, ``lib()`` raises.
"""
import ctypes
import os

from . import build as _build

c_double_p = ctypes.POINTER(ctypes.c_double)
c_void_p = ctypes.c_void_p
c_int = ctypes.c_int
c_i64 = ctypes.c_int64
c_size = ctypes.c_size_t

TT_OK = 0
TT_F32 = 0
TT_F64 = 1

RAY_OK = 0
RAY_STEP_TOO_SMALL = 1
RAY_MAX_STEPS = 2
RAY_NAN = 3

OPTIC_DISTANCE = 0
OPTIC_LENS = 1
OPTIC_CIRC_APERTURE = 2
OPTIC_CIRC_STOP = 3
OPTIC_ANNULUS_STOP = 4
OPTIC_RECT_APERTURE = 5
OPTIC_KNIFE_EDGE = 6
OPTIC_M_TO_MM = 7
MAX_OPTICS = 64
MAX_INSTANCES = 128
MAX_MARCH_FIELDS = 32


class TTError(RuntimeError):
    """A libturbotrace entry point returned a non-zero tt_status."""

    def __init__(self, status, where, detail):
        super().__init__("%s failed: %s (%s)" % (where, detail, status))
        self.status = status


class TTVolume(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32 * 3), ("axis", ctypes.c_int32 * 3), ("tiles", ctypes.c_int32 * 2),
                ("supertiles", ctypes.c_int32 * 2), ("bricks_c", ctypes.c_int32), ("brick_depth", ctypes.c_int32),
                ("origin", ctypes.c_double * 3), ("spacing", ctypes.c_double * 3), ("omega", ctypes.c_double),
                ("ne_max", ctypes.c_double), ("n_float4", ctypes.c_int64), ("nodes", ctypes.c_void_p)]


class TTTraceOpts(ctypes.Structure):
    _fields_ = [("rtol", ctypes.c_double), ("atol", ctypes.c_double), ("atol_phase", ctypes.c_double),
                ("max_steps", ctypes.c_int64), ("with_phase", ctypes.c_int32), ("block_size", ctypes.c_int32),
                ("ray_chunk", ctypes.c_int32), ("phase_f64", ctypes.c_int32), ("refill_lanes", ctypes.c_int32)]


TT_RK_MAX_STAGES = 16


class TTRKTableau(ctypes.Structure):
    _fields_ = [("n_stages", ctypes.c_int32), ("error_order", ctypes.c_int32), ("error_kind", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("A", (ctypes.c_double * TT_RK_MAX_STAGES) * TT_RK_MAX_STAGES),
                ("B", ctypes.c_double * TT_RK_MAX_STAGES), ("C", ctypes.c_double * TT_RK_MAX_STAGES),
                ("E", ctypes.c_double * (TT_RK_MAX_STAGES + 1)), ("E3", ctypes.c_double * (TT_RK_MAX_STAGES + 1))]


class TTFnoDims(ctypes.Structure):
    _fields_ = [("batch", ctypes.c_int32), ("size", ctypes.c_int32), ("in_ch", ctypes.c_int32),
                ("out_ch", ctypes.c_int32), ("layers", ctypes.c_int32)]


FNO_WIDTH = 32
FNO_MODES = 16
FNO_MAX_LAYERS = 8
FNO_MAX_IN = 16
FNO_MAX_OUT = 4


class TTOptic(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("reserved", ctypes.c_int32), ("p", ctypes.c_double * 3)]


# name -> (restype, argtypes); every symbol declared in include/turbotrace.h
SIGNATURES = {
    "tt_abi_version": (c_int, []),
    "tt_strerror": (ctypes.c_char_p, [c_int]),
    "tt_last_error_detail": (ctypes.c_char_p, []),
    "tt_calc_dndr_workspace_bytes": (c_size, [c_int, c_int, c_int]),
    "tt_calc_dndr": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                             ctypes.c_double, ctypes.c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                             c_double_p, c_void_p, c_size, c_void_p]),
    "tt_calc_dndr_noalloc": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                     ctypes.c_double, ctypes.c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                                     c_double_p, c_void_p]),
    "tt_dndr": (c_int, [ctypes.POINTER(c_void_p), c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                        c_void_p, c_i64, c_void_p, c_void_p]),
    "tt_volume_plan": (c_int, [c_int, c_int, c_int, c_double_p, c_double_p, c_double_p, c_int,
                               ctypes.c_double, ctypes.c_double, ctypes.POINTER(TTVolume)]),
    "tt_volume_set_brick_depth": (c_int, [ctypes.POINTER(TTVolume), c_int]),
    "tt_volume_build": (c_int, [ctypes.POINTER(TTVolume), c_void_p, c_int, c_void_p]),
    "tt_trace_f64": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p,
                             c_void_p, ctypes.c_double, c_void_p, c_i64, ctypes.c_double, c_int,
                             ctypes.c_double, ctypes.POINTER(TTTraceOpts), c_void_p, c_void_p, c_void_p,
                             c_void_p, c_void_p, c_void_p]),
    "tt_trace_f64_rk": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p,
                                c_void_p, ctypes.c_double, c_void_p, c_i64, ctypes.c_double, c_int,
                                ctypes.c_double, ctypes.POINTER(TTTraceOpts), ctypes.POINTER(TTRKTableau), c_void_p,
                                c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tt_trace_f32_workspace_bytes": (c_size, [ctypes.POINTER(TTVolume), c_i64]),
    "tt_trace_f32": (c_int, [ctypes.POINTER(TTVolume), c_void_p, c_i64, ctypes.c_double, ctypes.c_double,
                             ctypes.POINTER(TTTraceOpts), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                             c_void_p, c_size, c_void_p]),
    "tt_trace_f32_batched_workspace_bytes": (c_size, [ctypes.POINTER(TTVolume), c_int, c_i64]),
    "tt_trace_f32_batched": (c_int, [ctypes.POINTER(TTVolume), c_int, ctypes.POINTER(c_i64), c_double_p, c_double_p,
                                     c_void_p, ctypes.POINTER(TTTraceOpts), c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_void_p, c_void_p, c_size, c_void_p]),
    "tt_detect": (c_int, [c_void_p, c_i64, ctypes.POINTER(TTOptic), c_int, c_int, c_int, ctypes.c_double,
                          ctypes.c_double, ctypes.c_double, ctypes.c_double, c_void_p, c_void_p, c_void_p,
                          c_void_p, c_int, c_void_p]),
    "tt_grf_fft_workspace_bytes": (c_size, [c_int]),
    "tt_grf_fft": (c_int, [ctypes.c_uint64, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size,
                           c_void_p]),
    "tt_grf_fft_nd_workspace_bytes": (c_size, [c_int, c_int]),
    "tt_grf_fft_nd": (c_int, [ctypes.c_uint64, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size,
                              c_void_p]),
    "tt_cos_field": (c_int, [c_int, c_int, c_int, c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, c_int,
                             c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tt_grf_field_workspace_bytes": (c_size, [c_int]),
    "tt_grf_field": (c_int, [ctypes.c_uint64, c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                             ctypes.c_double, ctypes.c_double, ctypes.c_double, c_int, c_void_p, c_void_p,
                             c_size, c_void_p]),
    "tt_philox": (c_int, [ctypes.c_uint64, ctypes.c_uint32, c_i64, c_void_p, c_void_p]),
    "tt_straight_line_maps": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_double_p, c_double_p, c_double_p,
                                      ctypes.c_double, ctypes.c_double, c_int, c_int, c_void_p, c_void_p]),
    "tt_march_maps_workspace_bytes": (c_size, [c_int, c_int, c_int]),
    "tt_march_maps_batched_workspace_bytes": (c_size, [c_int, c_int, c_int, c_int]),
    "tt_march_maps_batched": (c_int, [ctypes.POINTER(c_void_p), c_int, c_int, c_int, c_int, c_int, c_double_p,
                                      c_double_p, c_double_p, ctypes.c_double, ctypes.c_double, c_int, c_void_p,
                                      c_void_p, c_size, c_void_p]),
    "tt_march_maps_batched_stride": (c_int, [ctypes.POINTER(c_void_p), c_int, c_int, c_int, c_int, c_int,
                                             c_double_p, c_double_p, c_double_p, ctypes.c_double, ctypes.c_double,
                                             c_int, c_int, c_void_p, c_void_p, c_size, c_void_p]),
    "tt_march_maps": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_double_p, c_double_p, c_double_p,
                              ctypes.c_double, ctypes.c_double, c_int, c_void_p, c_void_p, c_size, c_void_p]),
    "tt_shadowgram": (c_int, [c_void_p, c_int, ctypes.c_double, ctypes.c_double, c_void_p, c_void_p, c_void_p]),
    "tt_shadowgram_batched": (c_int, [c_void_p, c_int, c_int, ctypes.c_double, c_void_p, c_void_p, c_void_p]),
    "tt_surrogate_encode": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "tt_surrogate_decode": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p, c_void_p,
                                    c_void_p]),
    "tt_surrogate_estimate": (c_int, [c_void_p, c_void_p, c_int, c_int, ctypes.c_double, c_void_p, c_void_p]),
    "tt_fno_param_count": (c_size, [ctypes.POINTER(TTFnoDims)]),
    "tt_fno_workspace_bytes": (c_size, [ctypes.POINTER(TTFnoDims), c_int]),
    "tt_fno_forward": (c_int, [ctypes.POINTER(TTFnoDims), c_void_p, c_void_p, c_void_p, c_void_p, c_size, c_void_p]),
    "tt_fno_train_step": (c_int, [ctypes.POINTER(TTFnoDims), c_void_p, c_void_p, c_void_p, c_void_p,
                                  ctypes.POINTER(ctypes.c_float), c_void_p, c_void_p, c_void_p, c_size, c_void_p]),
    "tt_fno_adam": (c_int, [c_i64, c_void_p, c_void_p, c_void_p, c_void_p, ctypes.c_float, ctypes.c_float,
                            ctypes.c_float, ctypes.c_float, c_i64, c_void_p]),
    "tt_fno_adam_device": (c_int, [c_i64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, ctypes.c_float,
                                   ctypes.c_float, ctypes.c_float, c_void_p, c_void_p]),
    "tt_fno_error_flag": (c_int, [c_void_p, ctypes.POINTER(c_int)]),
    "tt_fno_pack": (c_int, [c_i64, c_int, c_void_p, c_void_p, c_void_p]),
    "tt_fno_rowdft": (c_int, [c_int, c_i64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tt_fno_mix": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                           c_void_p, c_void_p, c_void_p, c_void_p]),
    "tt_fno_wgrad": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tt_fno_rowdft_timeout_test": (c_int, [c_int, c_i64, c_void_p, c_void_p, c_void_p, c_void_p, c_i64, c_void_p]),
}

_lib = None


def library_path():
    return _build.LIB


def lib(build_if_missing=True):
    """Load libturbotrace.so (building it first if needed); raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libturbotrace.so is not built (expected %s); run "
                           "turbulence_tracing_gb300.build.build()" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status, where):
    if status != TT_OK:
        L = lib()
        detail = L.tt_last_error_detail().decode(errors="replace") or L.tt_strerror(status).decode()
        raise TTError(status, where, detail)
