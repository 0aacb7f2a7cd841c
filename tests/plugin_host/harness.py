"""Builds and calls the plugin host harness: the PLUMED plugin source
(plumed2_gb300/plugin/CoordinationGPU.cpp) compiled unchanged against the
minimal action interface in tests/plugin_host/include, with host.cpp stepping
one action through frames as `plumed driver` does.  Test infrastructure."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(HERE, "_build", "libplugin_host.so")
PLUGIN = os.path.join(ROOT, "plumed2_gb300", "plugin", "CoordinationGPU.cpp")
_lib = None


def build():
    from plumed2_gb300 import _lib as core
    core.load()  # libcoordgpu.so, built if missing
    libdir = os.path.dirname(core.LIB_PATH)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    srcs = [os.path.join(HERE, "host.cpp"), PLUGIN]
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) > os.path.getmtime(s) for s in srcs):
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I" + os.path.join(HERE, "include"),
           "-I" + os.path.join(ROOT, "include")] + srcs + ["-L" + libdir, "-lcoordgpu", "-Wl,-rpath," + libdir,
                                                          "-o", LIB]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("plugin host build failed:\n" + p.stderr)
    return LIB


def load():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        _dp = C.POINTER(C.c_double)
        L.plugin_host_run.argtypes = [C.c_char_p, C.c_longlong, C.c_int, C.c_longlong, _dp, _dp, _dp, _dp, _dp, _dp,
                                      C.POINTER(C.c_longlong), C.c_char_p, C.c_int, C.c_char_p, C.c_int]
        _lib = L
    return _lib


class PluginError(RuntimeError):
    pass


def run(line, frames, boxes, stride=1, charges=None):
    """Steps the action of `line` through frames [F][n_atoms][3] with boxes
    [F][3][3] (step = frame index x stride).  Returns values [F], derivatives
    by atom [F][n_atoms][3], box derivatives [F][3][3], requested atoms [F]
    and the action's log."""
    L = load()
    frames = np.ascontiguousarray(frames, dtype=np.float64)
    F, n = frames.shape[0], frames.shape[1]
    boxes = np.ascontiguousarray(np.asarray(boxes, dtype=np.float64).reshape(F, 9))
    q = None if charges is None else np.ascontiguousarray(np.broadcast_to(charges, (F, n)), dtype=np.float64)
    vals = np.zeros(F)
    der = np.zeros((F, n, 3))
    vir = np.zeros((F, 9))
    nreq = np.zeros(F, dtype=np.int64)
    log = C.create_string_buffer(1 << 16)
    err = C.create_string_buffer(4096)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    rc = L.plugin_host_run(line.encode(), n, F, stride, dp(frames), dp(boxes), dp(q) if q is not None else None,
                           dp(vals), dp(der), dp(vir), nreq.ctypes.data_as(C.POINTER(C.c_longlong)), log, len(log),
                           err, len(err))
    if rc != 0:
        raise PluginError(err.value.decode())
    return vals, der, vir.reshape(F, 3, 3), nreq, log.value.decode()
