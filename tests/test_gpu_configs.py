"""Parity at the benchmark configurations' own sizes (seeded synthetic frames
from plumed2_gb300.frames), against the C oracle:

* C1  32,768 atoms, GROUPA/GROUPB = the two z-slabs, RATIONAL R_0=0.35
      D_MAX=1.2, NLIST NL_CUTOFF=1.4 NL_STRIDE=20, three frames (the list of
      step 0 is reused, NeighborList::prepare); FP64 and mixed
* C2  100,000 atoms, 256 single-list actions (sizes log-uniform in [16, 4096],
      R_0 ~ U(0.25, 0.45), D_MAX=1.0, no list) in one fused batch; and the
      literal GROUPB=GROUPA form, which counts every pair twice
* C4  one 262,144-atom walker, NLIST NL_CUTOFF=0.8, mixed precision: the pair
      set bit-exact, s and forces within the mixed tolerance
Tolerances as in test_gpu_parity.py.
"""
import ctypes as C

import numpy as np
import pytest

from plumed2_gb300 import frames as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = {"fp64": (1e-12, 1e-11), "mixed": (1e-6, 1e-5)}


def _check(prec, got, ref, what=""):
    s, d, v = got
    s0, d0, v0 = ref
    ts, td = TOL[prec]
    assert abs(s - s0) <= ts * abs(s0), (what, s, s0)
    dscale = np.abs(d0).max()
    assert np.abs(d - d0).max() <= td * dscale, (what, np.abs(d - d0).max() / dscale)
    vscale = np.abs(v0).max()
    assert np.abs(v - v0).max() <= td * vscale, (what, np.abs(v - v0).max() / vscale)


def _sorted(p):
    p = np.asarray(p).reshape(-1, 2)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_c1_two_slab_groups(orc, prec):
    from plumed2_gb300.action import Coordination
    frames, box = W.workload_c1(n_frames=3)
    spec = "RATIONAL R_0=0.35 NN=6 MM=12 D_MAX=1.2"
    c = Coordination("GROUPA=1-16384 GROUPB=16385-32768 SWITCH={%s} NLIST NL_CUTOFF=1.4 NL_STRIDE=20" % spec,
                     precision=prec)
    nth = orc.max_threads()
    pairs = None
    for step, pos in enumerate(frames):
        got = c.calculate(pos, box, step)
        if step == 0:
            pairs = orc.nl_classic_cells(1, 16384, 16384, pos, box, True, 1.4)
            assert np.array_equal(_sorted(c.pairs()), pairs)
        ref = orc.coordination(spec, pos, box, pairs, nthreads=nth)
        _check(prec, got, ref, "C1 step %d" % step)
    c.close()


def test_c2_many_actions_batch(orc):
    from plumed2_gb300 import _lib
    from plumed2_gb300.action import Coordination
    pos, box = W.workload_c2_system()
    sizes, starts, r0 = W.workload_c2_actions(256)
    specs = ["RATIONAL R_0=%.6f NN=6 MM=12 D_MAX=1.0" % x for x in r0]
    acts = [Coordination("GROUPA=%d-%d SWITCH={%s}" % (st + 1, st + sz, sp), precision="mixed")
            for sz, st, sp in zip(sizes, starts, specs)]
    L = _lib.load()
    for a in acts:
        a._ensure_groups()
    arr = (C.c_void_p * len(acts))(*[a._ctx.value for a in acts])
    m = C.c_void_p()
    assert L.coord_multi_create(arr, len(acts), len(pos), C.byref(m)) == 0, L.coord_multi_last_error(m)
    offs = []
    per = C.c_int64()
    for k in range(len(acts)):
        o = C.c_int64()
        assert L.coord_multi_deriv_offset(m, k, C.byref(o), C.byref(per)) == 0
        offs.append(o.value)
    dev = torch.device("cuda:0")
    tpos = torch.tensor(pos[None], dtype=torch.float64, device=dev)
    s = torch.zeros(1, len(acts), dtype=torch.float64, device=dev)
    der = torch.zeros(1, per.value, dtype=torch.float64, device=dev)
    vir = torch.zeros(1, len(acts), 9, dtype=torch.float64, device=dev)
    bx = np.ascontiguousarray(box.reshape(1, 9))
    torch.cuda.synchronize()
    rc = L.coord_multi_forward_device(m, 1, C.c_void_p(tpos.data_ptr()), bx.ctypes.data_as(C.POINTER(C.c_double)), 0,
                                      C.c_void_p(s.data_ptr()), C.c_void_p(der.data_ptr()),
                                      C.c_void_p(vir.data_ptr()), None)
    assert rc == 0, L.coord_multi_last_error(m)
    torch.cuda.synchronize()
    S, D, V = s.cpu().numpy()[0], der.cpu().numpy()[0], vir.cpu().numpy()[0]
    # every action's s; derivatives and virial for a sample (incl. the largest)
    rng = np.random.default_rng(9)
    sample = set(rng.choice(len(acts), 24, replace=False).tolist()) | {int(np.argmax(sizes))}
    nth = orc.max_threads()
    for k in range(len(acts)):
        sz, st = int(sizes[k]), int(starts[k])
        sub = pos[st:st + sz]
        ref = orc.coordination(specs[k], sub, box, orc.all_pairs(0, sz), nthreads=nth)
        assert abs(S[k] - ref[0]) <= 1e-6 * abs(ref[0]), (k, S[k], ref[0])
        if k in sample:
            d1 = D[offs[k]:offs[k] + 3 * sz].reshape(sz, 3)
            _check("mixed", (S[k], d1, V[k].reshape(3, 3)), ref, "C2 action %d" % k)
    L.coord_multi_destroy(m)
    for a in acts:
        a.close()


def test_c2_groupb_equals_groupa_counts_twice():
    from plumed2_gb300.action import Coordination
    pos, box = W.workload_c2_system()
    spec = "RATIONAL R_0=0.31 NN=6 MM=12 D_MAX=1.0"
    for lo, hi in ((5001, 5600), (70001, 70040)):
        one = Coordination("GROUPA=%d-%d SWITCH={%s}" % (lo, hi, spec))
        two = Coordination("GROUPA=%d-%d GROUPB=%d-%d SWITCH={%s}" % (lo, hi, lo, hi, spec))
        s1, d1, v1 = one.calculate(pos[lo - 1:hi], box)
        s2, d2, v2 = two.calculate(np.concatenate([pos[lo - 1:hi], pos[lo - 1:hi]]), box)
        assert abs(s2 - 2 * s1) <= 1e-12 * abs(s1)
        n = hi - lo + 1
        np.testing.assert_allclose(d2[:n] + d2[n:], 2 * d1, rtol=0, atol=1e-11 * np.abs(d1).max())
        np.testing.assert_allclose(v2, 2 * v1, rtol=0, atol=1e-11 * np.abs(v1).max())


def test_c4_walker_pair_set_and_values(orc):
    from plumed2_gb300.action import Coordination
    pos, box = W.workload_c4_walker(0)
    n = len(pos)
    spec = "RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.6"
    c = Coordination("GROUPA=1-%d SWITCH={%s} NLIST NL_CUTOFF=0.8 NL_STRIDE=10" % (n, spec), precision="mixed")
    got = c.calculate(pos, box, 0)
    pairs = orc.nl_classic_cells(0, n, 0, pos, box, True, 0.8)
    assert c.nl_size() == len(pairs)
    assert np.array_equal(_sorted(c.pairs()), pairs)
    ref = orc.coordination(spec, pos, box, pairs, nthreads=orc.max_threads())
    _check("mixed", got, ref, "C4 walker 0")
    c.close()
