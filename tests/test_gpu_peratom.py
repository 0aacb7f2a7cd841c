"""Per-atom coordination (COORDINATIONNUMBER = CONTACT_MATRIX x ones) on the
GPU against the reference's regtest goldens and the FP64 oracle.

Tolerances:
  goldens   the print format (%.4f, %8.4f)
  FP64      cn: max|dcn| <= 1e-12 max|cn|; backward: max|d| <= 1e-11 max|ref|
  mixed     cn: max|dcn| <= 2e-6 max|cn| (FP32 pair math and FP32 per-atom
            sums); backward: max|d| <= 1e-5 max|ref| (the force bound of the
            mixed path)
"""
import numpy as np
import pytest

from plumed2_gb300.frames import jittered_lattice

pytestmark = pytest.mark.gpu

TOL = {"fp64": (1e-12, 1e-11), "mixed": (2e-6, 1e-5)}


def test_rt_dumpmulti_golden(golden):
    from plumed2_gb300.action import CoordinationNumbers
    d = golden("rt_peratom.json")["dumpmulti"]
    c = CoordinationNumbers("SPECIES=%s SWITCH={%s}" % (d["species"], d["spec"]))
    cn = c.calculate(np.array(d["pos"]), np.diag(d["box"]))
    assert np.abs(cn - np.array(d["cn"])).max() <= 5.01e-5


def test_rt_single_groupb_golden(golden):
    from plumed2_gb300.action import CoordinationNumbers
    g = golden("rt_peratom.json")["single_groupb"]
    c = CoordinationNumbers("SPECIESA=%s SPECIESB=%s SWITCH={%s}" % (g["speciesa"], g["speciesb"], g["spec"]))
    for fi, (fr, bx) in enumerate(zip(g["frames"], g["box"])):
        cn = c.calculate(np.array(fr), np.diag(bx), step=fi)
        assert np.abs(cn - np.array(g["cn"][fi])).max() <= 5.01e-5, fi


def _device(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda:0")


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("groups", ["species", "ab"])
def test_peratom_parity_and_vjp(orc, prec, groups):
    """cn and the vector-Jacobian product against the oracle over the same
    pairs (a list with cutoff d_max), batched over two frames."""
    import torch
    from plumed2_gb300.action import CoordinationNumbers
    spec = "RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.75"
    n, F = 1500, 2
    frames = np.stack([jittered_lattice(n, 0.31, 0.04, 40 + f) for f in range(F)])
    L = 0.31 * round(n ** (1 / 3) + 0.5)
    boxes = np.stack([np.diag([L] * 3)] * F)
    if groups == "species":
        c = CoordinationNumbers("SPECIES=1-%d SWITCH={%s}" % (n, spec), precision=prec)
        m, n0, n1 = 0, n, 0
    else:
        c = CoordinationNumbers("SPECIESA=1-600 SPECIESB=601-%d SWITCH={%s}" % (n, spec), precision=prec)
        m, n0, n1 = 1, 600, n - 600
    pos = _device(frames)
    cn = torch.empty(F, n, dtype=torch.float64, device=pos.device)
    c.forward_device(pos.data_ptr(), boxes, F, cn.data_ptr())
    rng = np.random.default_rng(3)
    g = rng.uniform(-1.0, 1.0, (F, n))
    gd = _device(g)
    gpos = torch.empty(F, n, 3, dtype=torch.float64, device=pos.device)
    gbox = torch.empty(F, 9, dtype=torch.float64, device=pos.device)
    c.backward_device(pos.data_ptr(), boxes, F, gd.data_ptr(), gpos.data_ptr(), gbox.data_ptr())
    tc, tb = TOL[prec]
    cn, gpos, gbox = cn.cpu().numpy(), gpos.cpu().numpy(), gbox.cpu().numpy()
    for f in range(F):
        pairs = orc.nl_classic(m, n0, n1, frames[f], boxes[f], True, 0.75)
        rcn, rgrad, rvir = orc.peratom(spec, frames[f], boxes[f], pairs, g=g[f])
        assert np.abs(cn[f] - rcn).max() <= tc * np.abs(rcn).max(), (f, np.abs(cn[f] - rcn).max())
        assert np.abs(gpos[f] - rgrad).max() <= tb * np.abs(rgrad).max(), (f, np.abs(gpos[f] - rgrad).max())
        # dV/dh with scaled coordinates fixed: -(invBox^T) applied to the virial
        inv = np.linalg.inv(boxes[f])
        rgb = -(inv.T @ rvir)
        assert np.abs(gbox[f].reshape(3, 3) - rgb).max() <= tb * np.abs(rgb).max(), f


def test_peratom_nlistcells_context(orc):
    """The C call on a COORDINATION context with NLISTCELLS: the link cells'
    superset of pairs gives the same sums (pairs beyond d_max weigh 0)."""
    import torch
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.75"
    n = 1000
    pos = jittered_lattice(n, 0.31, 0.04, 9)
    box = np.diag([3.1] * 3)
    c = Coordination("GROUPA=1-%d SWITCH={%s} NLISTCELLS NL_CUTOFF=0.75 NL_STRIDE=1" % (n, spec))
    c._ensure_groups()
    p = _device(pos.reshape(1, n, 3))
    cn = torch.empty(1, n, dtype=torch.float64, device=p.device)
    from plumed2_gb300._lib import check
    import ctypes as C
    from plumed2_gb300._lib import dptr
    bx = np.ascontiguousarray(box.reshape(1, 9))
    check(c._L, c._ctx, c._L.coord_peratom_device(c._ctx, 1, C.c_void_p(p.data_ptr()), dptr(bx), 0, 0,
                                                    C.c_void_p(cn.data_ptr()), None, None))
    ref = orc.peratom(spec, pos, box, orc.nl_linkcells(0, n, 0, pos, box, True, 0.75))
    assert np.abs(cn.cpu().numpy()[0] - ref).max() <= 1e-12 * np.abs(ref).max()


def test_peratom_autograd_finite_differences():
    """V = sum_i w_i cn_i^2 through torch autograd against FP64 central
    differences (h = 1e-6 nm) of the forward, for positions and the box."""
    import torch
    from plumed2_gb300.action import CoordinationNumbers
    from plumed2_gb300.autograd import coordination_numbers
    n = 343
    x = jittered_lattice(n, 0.3, 0.04, 17)
    box0 = np.diag([2.1] * 3)
    c = CoordinationNumbers("SPECIES=1-%d SWITCH={RATIONAL R_0=0.3 D_MAX=0.7}" % n)
    w = torch.as_tensor(np.random.default_rng(4).uniform(0.5, 1.5, n), device="cuda:0")

    def V(xx, bb):
        cn = coordination_numbers(c, torch.as_tensor(xx, device="cuda:0"), torch.as_tensor(bb))
        return (w * cn * cn).sum()

    pos = torch.as_tensor(x, device="cuda:0").requires_grad_(True)
    box = torch.as_tensor(box0).requires_grad_(True)
    V(pos, box).backward()
    h = 1e-6
    for i, k in [(0, 0), (17, 1), (200, 2), (342, 0)]:
        xp, xm = x.copy(), x.copy()
        xp[i, k] += h
        xm[i, k] -= h
        fd = (V(xp, box0).item() - V(xm, box0).item()) / (2 * h)
        assert abs(pos.grad[i, k].item() - fd) <= 1e-6 * max(1.0, abs(fd)), (i, k, pos.grad[i, k].item(), fd)
    # box derivative with scaled coordinates fixed
    for a, b in [(0, 0), (1, 1), (2, 2)]:
        bp, bm = box0.copy(), box0.copy()
        bp[a, b] += h
        bm[a, b] -= h
        sp = x @ np.linalg.inv(box0) @ bp
        sm = x @ np.linalg.inv(box0) @ bm
        fd = (V(sp, bp).item() - V(sm, bm).item()) / (2 * h)
        assert abs(box.grad[a, b].item() - fd) <= 1e-5 * max(1.0, abs(fd)), (a, b, box.grad[a, b].item(), fd)


def test_peratom_refusals():
    import ctypes as C
    from plumed2_gb300 import _lib
    from plumed2_gb300.action import Coordination, CoordinationNumbers, DHEnergy
    with pytest.raises(ValueError, match="SPECIES"):
        CoordinationNumbers("SWITCH={RATIONAL R_0=1}")
    with pytest.raises(ValueError, match="SWITCH/R_0"):
        CoordinationNumbers("SPECIES=1-10")
    import torch
    box = np.ascontiguousarray(np.eye(3).reshape(1, 9))
    pos = torch.zeros(1, 10, 3, dtype=torch.float64, device="cuda:0")
    cn = torch.zeros(1, 10, dtype=torch.float64, device="cuda:0")
    for act in (Coordination("GROUPA=1-10 R_0=0.3"), Coordination("PAIR GROUPA=1-5 GROUPB=6-10 R_0=0.3 NLIST "
                                                                  "NL_CUTOFF=1 NL_STRIDE=1"),
                DHEnergy("GROUPA=1-10 NLIST NL_CUTOFF=1 NL_STRIDE=1")):
        act._ensure_groups()
        rc = act._L.coord_peratom_device(act._ctx, 1, C.c_void_p(pos.data_ptr()), _lib.dptr(box), 0, 0,
                                         C.c_void_p(cn.data_ptr()), None, None)
        assert rc == _lib.COORD_ERR_UNSUPPORTED
