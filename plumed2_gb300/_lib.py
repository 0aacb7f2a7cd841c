"""ctypes binding of libcoordgpu.so (the C ABI declared in include/coordgpu.h).

The library is loaded from plumed2_gb300/_build/.  There is no fallback:
when the library is missing, building it is attempted once and any failure
is raised to the caller.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcoordgpu.so")

COORD_OK = 0
COORD_ERR_ARG = 1
COORD_ERR_CUDA = 2
COORD_ERR_BOX = 3
COORD_ERR_UNSUPPORTED = 4
COORD_ERR_NOMEM = 5
COORD_ERR_TIMEOUT = 6
COORD_ERR_STATE = 7

NL_NONE, NL_CLASSIC, NL_CELLS = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
CV_COORDINATION, CV_DHENERGY, CV_GHBFIX = 0, 1, 2
CMAP_COMPONENTS, CMAP_SUM, CMAP_CMDIST = 0, 1, 2
FLAG_REBUILD, FLAG_NO_DERIV, FLAG_DR0, FLAG_SAVE = 1, 2, 4, 8


class CoordParams(C.Structure):
    _fields_ = [("switch_def", C.c_char_p), ("r0", C.c_double), ("d0", C.c_double), ("nn", C.c_int),
                ("mm", C.c_int), ("nopbc", C.c_int), ("pair", C.c_int), ("nlist", C.c_int),
                ("nl_cutoff", C.c_double), ("nl_stride", C.c_int), ("serial", C.c_int), ("precision", C.c_int),
                ("device", C.c_int)]


class CoordError(RuntimeError):
    """A nonzero status of the C ABI, with coord_last_error()'s message."""

    def __init__(self, status: int, message: str):
        super().__init__("%s (status %d: %s)" % (message, status, _STATUS.get(status, "?")))
        self.status = status
        self.message = message


_STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "invalid box", 4: "unsupported input",
           5: "out of device memory", 6: "device wait timed out", 7: "call out of order"}

_lock = threading.Lock()
_lib = None

_vp = C.c_void_p
_dp = C.POINTER(C.c_double)


def load() -> C.CDLL:
    """Load (building if needed) libcoordgpu.so and declare its signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            from . import build as _build
            _build.build()
        L = C.CDLL(LIB_PATH)
        L.coord_params_default.argtypes = [C.POINTER(CoordParams)]
        L.coord_params_default.restype = None
        L.coord_create.argtypes = [C.POINTER(CoordParams), C.POINTER(_vp)]
        L.coord_destroy.argtypes = [_vp]
        L.coord_last_error.argtypes = [_vp]
        L.coord_last_error.restype = C.c_char_p
        L.coord_status_string.argtypes = [C.c_int]
        L.coord_status_string.restype = C.c_char_p
        L.coord_set_groups.argtypes = [_vp, C.POINTER(C.c_int64), C.c_int64, C.POINTER(C.c_int64), C.c_int64]
        L.coord_get_nslots.argtypes = [_vp, C.POINTER(C.c_int64)]
        L.coord_set_dhenergy.argtypes = [_vp] + [C.c_double] * 6
        L.coord_set_charges.argtypes = [_vp, _dp, C.c_int64]
        L.coord_forward_batch.argtypes = [_vp, C.c_int, _vp, _vp, C.c_int64, C.c_uint, _vp, _vp, _vp]
        L.coord_cmap_create.argtypes = [C.c_int64, C.POINTER(C.c_char_p), C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_int,
                                        C.POINTER(_vp)]
        L.coord_cmap_destroy.argtypes = [_vp]
        L.coord_cmap_last_error.argtypes = [_vp]
        L.coord_cmap_last_error.restype = C.c_char_p
        L.coord_cmap_forward_device.argtypes = [_vp, C.c_int, _vp, _dp, _vp, _vp, _vp, _vp]
        L.coord_peratom_device.argtypes = [_vp, C.c_int, _vp, _dp, C.c_int64, C.c_uint, _vp, _vp, _vp]
        L.coord_peratom_backward_device.argtypes = [_vp, C.c_int, _vp, _dp, _vp, _vp, _vp, _vp]
        L.coord_set_ghbfix.argtypes = [_vp, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_int32), C.c_int64, _dp,
                                       C.c_int]
        L.coord_switch_eval.argtypes = [_vp, C.c_int, _dp, C.c_int, _dp, _dp]
        L.coord_switch_params.argtypes = [_vp, _dp]
        L.coord_forward.argtypes = [_vp, _dp, _dp, C.c_int64, C.c_uint, _dp, _dp, _dp]
        # the same entry with plain addresses (integers), as a compiled caller passes them
        L.coord_forward_addr = L["coord_forward"]
        L.coord_forward_addr.argtypes = [_vp, _vp, _vp, C.c_int64, C.c_uint, _vp, _vp, _vp]
        L.coord_forward_addr.restype = C.c_int
        L.coord_forward_device.argtypes = [_vp, C.c_int, _vp, _dp, C.c_int64, C.c_uint, _vp, _vp, _vp, _vp, _vp]
        L.coord_backward_device.argtypes = [_vp, C.c_int, _vp, _dp, _vp, _vp, _vp, _vp, _vp]
        L.coord_nl_size.argtypes = [_vp, C.c_int, C.POINTER(C.c_int64)]
        L.coord_nl_near_size.argtypes = [_vp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_double)]
        L.coord_get_pairs.argtypes = [_vp, C.c_int, C.POINTER(C.c_uint32), C.c_int64, C.POINTER(C.c_int64)]
        L.coord_multi_create.argtypes = [C.POINTER(_vp), C.c_int, C.c_int64, C.POINTER(_vp)]
        L.coord_multi_destroy.argtypes = [_vp]
        L.coord_multi_deriv_offset.argtypes = [_vp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.coord_multi_forward_device.argtypes = [_vp, C.c_int, _vp, _dp, C.c_uint, _vp, _vp, _vp, _vp]
        L.coord_multi_use_graph.argtypes = [_vp, C.c_int]
        L.coord_multi_last_error.argtypes = [_vp]
        L.coord_multi_last_error.restype = C.c_char_p
        L.coord_autotune.argtypes = [_vp, C.c_char_p, C.c_size_t]
        L.coord_measure_peaks.argtypes = [C.c_int, _dp, _dp, _dp]
        L.coord_launch_count.restype = C.c_int64
        L.coord_last_kernel_ms.argtypes = [_vp, _dp, C.POINTER(C.c_int)]
        L.coord_set_timing.argtypes = [_vp, C.c_int]
        L.coord_kernel_times.argtypes = [_vp, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_int)]
        L.coord_host_memory_access.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.coord_host_path.argtypes = [_vp]
        L.coord_apply_forces.argtypes = [_vp, C.c_int, _vp, C.c_int64, _vp, _vp, _vp]
        L.coord_bias_hills.argtypes = [C.c_int, _vp, C.c_int, _vp, _vp, _vp, C.c_int, C.c_int, _vp, _vp, _vp]
        L.coord_bias_restraint.argtypes = [C.c_int, _vp, C.c_double, C.c_double, C.c_double, C.c_int, _vp, _vp, _vp]
        L.coord_forward_noalloc.argtypes = [_vp, C.POINTER(C.c_int64), C.c_int64, C.POINTER(C.c_int64), C.c_int64,
                                            _vp, _dp, _vp, _vp, _vp, _vp]
        _lib = L
        return L


def dptr(a: np.ndarray):
    return C.cast(a.__array_interface__["data"][0], _dp)


def addr(a: np.ndarray) -> int:
    """Address of a numpy array's first element."""
    return a.__array_interface__["data"][0]


def check(L, ctx, rc: int):
    if rc != COORD_OK:
        msg = L.coord_last_error(ctx).decode() if ctx else _STATUS.get(rc, "")
        raise CoordError(rc, msg)


def measure_peaks(device: int = 0):
    L = load()
    f32, f64, hbm = C.c_double(), C.c_double(), C.c_double()
    rc = L.coord_measure_peaks(device, C.byref(f32), C.byref(f64), C.byref(hbm))
    if rc:
        raise CoordError(rc, "coord_measure_peaks")
    return {"fp32_tflops": f32.value, "fp64_tflops": f64.value, "hbm_gbs": hbm.value}


def launch_count() -> int:
    return int(load().coord_launch_count())


def host_memory_access(device: int = 0):
    """(pageable, via host page tables): whether kernels can access the caller's host arrays directly."""
    a, b = C.c_int(), C.c_int()
    load().coord_host_memory_access(device, C.byref(a), C.byref(b))
    return bool(a.value), bool(b.value)


def bias_hills(n_frames: int, s_ptr: int, n_hills: int, centers_ptr: int, sigmas_ptr: int, heights_ptr: int,
               V_ptr: int = 0, dVds_ptr: int = 0, stretch: bool = True, accumulate: bool = False, stream: int = 0):
    """Truncated Gaussian hills on the device (coord_bias_hills); pointers are device addresses."""
    rc = load().coord_bias_hills(int(n_frames), C.c_void_p(s_ptr), int(n_hills), C.c_void_p(centers_ptr),
                                 C.c_void_p(sigmas_ptr), C.c_void_p(heights_ptr), int(bool(stretch)),
                                 int(bool(accumulate)), C.c_void_p(V_ptr or None), C.c_void_p(dVds_ptr or None),
                                 C.c_void_p(stream or None))
    if rc:
        raise CoordError(rc, "coord_bias_hills")


def bias_restraint(n_frames: int, s_ptr: int, at: float, kappa: float, slope: float = 0.0, V_ptr: int = 0,
                   dVds_ptr: int = 0, accumulate: bool = False, stream: int = 0):
    """RESTRAINT on the device (coord_bias_restraint); pointers are device addresses."""
    rc = load().coord_bias_restraint(int(n_frames), C.c_void_p(s_ptr), float(at), float(kappa), float(slope),
                                     int(bool(accumulate)), C.c_void_p(V_ptr or None), C.c_void_p(dVds_ptr or None),
                                     C.c_void_p(stream or None))
    if rc:
        raise CoordError(rc, "coord_bias_restraint")
