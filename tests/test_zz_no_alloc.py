"""coord_forward_noalloc: the forward for callers that cannot allocate device
memory (an MD engine that reserves its whole device pool up front) must give
the same answer as the ordinary entry point.

Called through the C ABI on two calls in a row (different positions, so the
second call also shows that the shared static scratch is cleared between
calls), against coord_forward on the same inputs.  Tolerance: the FP64 one of
the other GPU tests (s: 1e-12 relative; derivatives and virial: 1e-11 of the
largest magnitude).  Collected last (file name) so a failure here stops a run
only after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from plumed2_gb300.frames import jittered_lattice

pytestmark = pytest.mark.gpu


def test_noalloc_matches_existing_entry_point():
    torch = pytest.importorskip("torch")
    from plumed2_gb300 import _lib
    from plumed2_gb300.action import Coordination

    L = _lib.load()
    dev = torch.device("cuda:0")
    torch.cuda.set_device(0)
    spec = "RATIONAL R_0=0.35 NN=6 MM=12 D_MAX=1.2"
    line_a, line_b = "1-700", "401-1000"
    system = [jittered_lattice(1000, 0.31, 0.03, 90), jittered_lattice(1000, 0.31, 0.03, 91)]
    box = np.diag([3.1, 3.1, 3.1])

    # the ordinary entry point
    ref = Coordination("GROUPA=%s GROUPB=%s SWITCH={%s}" % (line_a, line_b, spec))
    # a context for the no-allocation call: coord_create only (no coord_set_groups)
    p = _lib.CoordParams()
    L.coord_params_default(C.byref(p))
    sw = spec.encode()
    p.switch_def = sw
    ctx = C.c_void_p()
    assert L.coord_create(C.byref(p), C.byref(ctx)) == 0
    ga = np.ascontiguousarray(ref.group_a, dtype=np.int64)
    gb = np.ascontiguousarray(ref.group_b, dtype=np.int64)
    ns = len(ga) + len(gb)
    bx = np.ascontiguousarray(box.reshape(9))
    try:
        for call in range(2):
            pos = system[call][ref.requested_atoms]
            s0, d0, v0 = ref.calculate(pos, box, call)
            tpos = torch.tensor(pos, dtype=torch.float64, device=dev)
            s = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
            der = torch.full((ns, 3), 7.0, dtype=torch.float64, device=dev)
            vir = torch.full((9,), 7.0, dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            rc = L.coord_forward_noalloc(ctx, ga.ctypes.data_as(C.POINTER(C.c_int64)), len(ga),
                                         gb.ctypes.data_as(C.POINTER(C.c_int64)), len(gb),
                                         C.c_void_p(tpos.data_ptr()), bx.ctypes.data_as(C.POINTER(C.c_double)),
                                         C.c_void_p(s.data_ptr()), C.c_void_p(der.data_ptr()),
                                         C.c_void_p(vir.data_ptr()), None)
            assert rc == 0, L.coord_last_error(ctx).decode()
            torch.cuda.synchronize()
            s1, d1, v1 = s.item(), der.cpu().numpy(), vir.cpu().numpy().reshape(3, 3)
            assert abs(s1 - s0) <= 1e-12 * abs(s0), (call, s1, s0)
            assert np.abs(d1 - d0).max() <= 1e-11 * np.abs(d0).max(), call
            assert np.abs(v1 - v0).max() <= 1e-11 * np.abs(v0).max(), call
        # sizes beyond the fixed scratch are refused with a message
        big = np.arange(40000, dtype=np.int64)
        rc = L.coord_forward_noalloc(ctx, big.ctypes.data_as(C.POINTER(C.c_int64)), len(big), None, 0,
                                     C.c_void_p(tpos.data_ptr()), bx.ctypes.data_as(C.POINTER(C.c_double)),
                                     C.c_void_p(s.data_ptr()), C.c_void_p(der.data_ptr()), C.c_void_p(vir.data_ptr()),
                                     None)
        assert rc == _lib.COORD_ERR_ARG
        assert b"COORD_NOALLOC_MAX_SLOTS" in L.coord_last_error(ctx)
    finally:
        L.coord_destroy(ctx)
        ref.close()
