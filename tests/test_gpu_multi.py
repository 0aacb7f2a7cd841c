"""Many COORDINATION actions over one system in one batch (coord_multi_*).

Each action's s, derivatives and virial from the batch equal the action's own
single-context result: fused actions (mixed, no NLIST) within the mixed
tolerance of test_gpu_parity (s 1e-6 relative, derivatives/virial 1e-5 of
scale), actions run through their own context (FP64, NLIST) exactly.  Replays
of the captured CUDA graph give the same answers for new positions.
"""
import ctypes as C

import numpy as np
import pytest

from plumed2_gb300.frames import jittered_lattice

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _batch(acts, n_atoms):
    from plumed2_gb300 import _lib
    L = _lib.load()
    for a in acts:
        a._ensure_groups()
    arr = (C.c_void_p * len(acts))(*[a._ctx.value for a in acts])
    m = C.c_void_p()
    rc = L.coord_multi_create(arr, len(acts), n_atoms, C.byref(m))
    assert rc == 0, L.coord_multi_last_error(m)
    return L, m


def _offsets(L, m, n):
    offs = []
    per = C.c_int64()
    for k in range(n):
        o = C.c_int64()
        assert L.coord_multi_deriv_offset(m, k, C.byref(o), C.byref(per)) == 0
        offs.append(o.value)
    return offs, per.value


def test_multi_matches_single_contexts():
    from plumed2_gb300.action import Coordination
    dev = torch.device("cuda:0")
    n_atoms, L_box, F = 12167, 23 * 0.31, 3
    rng = np.random.default_rng(4)
    frames = np.stack([jittered_lattice(n_atoms, 0.31, 0.03, 200 + f) for f in range(F)])
    box = np.diag([L_box] * 3)
    acts, lines = [], []
    for k in range(14):
        size = int(np.exp(rng.uniform(np.log(16), np.log(1500))))
        start = int(rng.integers(0, n_atoms - size))
        r0 = rng.uniform(0.25, 0.45)
        if k % 5 == 4:
            line = "GROUPA=%d-%d GROUPB=%d-%d SWITCH={RATIONAL R_0=%.4f NN=6 MM=12 D_MAX=1.0}" % (
                start + 1, start + size // 2, start + size // 2 + 1, start + size, r0)
        else:
            line = "GROUPA=%d-%d SWITCH={RATIONAL R_0=%.4f NN=6 MM=12 D_MAX=1.0}" % (start + 1, start + size, r0)
        prec = "mixed"
        if k == 3:
            prec = "fp64"  # runs through its own context inside the batch
        if k == 6:
            line += " NLIST NL_CUTOFF=1.2 NL_STRIDE=5"
        acts.append(Coordination(line, precision=prec))
        lines.append((line, prec))
    Lb, m = _batch(acts, n_atoms)
    offs, per = _offsets(Lb, m, len(acts))
    tpos = torch.tensor(frames, dtype=torch.float64, device=dev)
    s = torch.zeros(F, len(acts), dtype=torch.float64, device=dev)
    der = torch.zeros(F, per, dtype=torch.float64, device=dev)
    vir = torch.zeros(F, len(acts), 9, dtype=torch.float64, device=dev)
    boxes = np.ascontiguousarray(np.stack([box] * F).reshape(F, 9))
    torch.cuda.synchronize()
    rc = Lb.coord_multi_forward_device(m, F, C.c_void_p(tpos.data_ptr()), boxes.ctypes.data_as(C.POINTER(C.c_double)),
                                       0, C.c_void_p(s.data_ptr()), C.c_void_p(der.data_ptr()),
                                       C.c_void_p(vir.data_ptr()), None)
    assert rc == 0, Lb.coord_multi_last_error(m)
    torch.cuda.synchronize()
    S, D, V = s.cpu().numpy(), der.cpu().numpy(), vir.cpu().numpy()
    for k, (line, prec) in enumerate(lines):
        ref = Coordination(line, precision=prec)
        for f in range(F):
            s0, d0, v0 = ref.calculate(frames[f][ref.requested_atoms], box, 0, rebuild=True)
            ns = ref.nslots
            d1 = D[f, offs[k]:offs[k] + 3 * ns].reshape(ns, 3)
            tol = 1e-12 if prec == "fp64" else 1e-6
            tol_d = 1e-11 if prec == "fp64" else 1e-5
            assert abs(S[f, k] - s0) <= tol * abs(s0) + 1e-12, (k, f, S[f, k], s0)
            assert np.abs(d1 - d0).max() <= tol_d * max(np.abs(d0).max(), 1e-12), (k, f)
            assert np.abs(V[f, k].reshape(3, 3) - v0).max() <= tol_d * max(np.abs(v0).max(), 1e-12), (k, f)
        ref.close()
    Lb.coord_multi_destroy(m)


def test_multi_graph_replay():
    from plumed2_gb300.action import Coordination
    dev = torch.device("cuda:0")
    n_atoms, L_box, F = 8000, 20 * 0.31, 2
    box = np.diag([L_box] * 3)
    acts = [Coordination("GROUPA=%d-%d SWITCH={RATIONAL R_0=0.3%d NN=6 MM=12 D_MAX=1.0}" % (1 + 300 * k, 300 * k + 250 + 40 * k, k),
                         precision="mixed") for k in range(8)]
    Lb, m = _batch(acts, n_atoms)
    assert Lb.coord_multi_use_graph(m, 1) == 0
    offs, per = _offsets(Lb, m, len(acts))
    tpos = torch.zeros(F, n_atoms, 3, dtype=torch.float64, device=dev)
    s = torch.zeros(F, len(acts), dtype=torch.float64, device=dev)
    der = torch.zeros(F, per, dtype=torch.float64, device=dev)
    vir = torch.zeros(F, len(acts), 9, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream()
    for call in range(3):
        frames = np.stack([jittered_lattice(n_atoms, 0.31, 0.03, 300 + 10 * call + f) for f in range(F)])
        boxes = np.ascontiguousarray(np.stack([box] * F).reshape(F, 9))
        tpos.copy_(torch.tensor(frames, dtype=torch.float64))
        torch.cuda.synchronize()
        rc = Lb.coord_multi_forward_device(m, F, C.c_void_p(tpos.data_ptr()),
                                           boxes.ctypes.data_as(C.POINTER(C.c_double)), 0, C.c_void_p(s.data_ptr()),
                                           C.c_void_p(der.data_ptr()), C.c_void_p(vir.data_ptr()),
                                           C.c_void_p(stream.cuda_stream))
        assert rc == 0, Lb.coord_multi_last_error(m)
        stream.synchronize()
        for k, a in enumerate(acts):
            for f in range(F):
                s0, d0, _ = a.calculate(frames[f][a.requested_atoms], box, 0)
                d1 = der[f, offs[k]:offs[k] + 3 * a.nslots].cpu().numpy().reshape(-1, 3)
                assert abs(s[f, k].item() - s0) <= 1e-6 * abs(s0), (call, k, f)
                assert np.abs(d1 - d0).max() <= 1e-5 * np.abs(d0).max(), (call, k, f)
    Lb.coord_multi_destroy(m)
