"""Backward pass: dV/dx, dV/dh (box), dV/dR_0, dV/dD_0 of a metadynamics-style
bias V(s) = sum_k h exp(-(s - s_k)^2 / (2 sigma^2)).

Checks, on the FP64 path:
  * against the oracle's analytic derivatives times V'(s) (the reference's
    own derivative layout): max|d| / max|ref| <= 1e-10
  * against FP64 central finite differences, step 1e-6 nm (positions; box
    with scaled coordinates held fixed) and 1e-6 nm in R_0/D_0:
    relative error <= 2e-6 of the gradient's scale
The mixed path's gradients against the FP64 path's: <= 1e-5 (norm-wise).
"""
import numpy as np
import pytest

from plumed2_gb300.frames import jittered_lattice

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def bias(s, s0):
    rng = np.random.default_rng(3)
    centres = torch.tensor(rng.uniform(0.8 * s0, 1.2 * s0, 500), dtype=torch.float64, device=s.device)
    sig = 0.05 * s0
    return (1.2 * torch.exp(-(s[:, None] - centres[None, :]) ** 2 / (2 * sig * sig))).sum(1)


def bias_np(s, s0):
    rng = np.random.default_rng(3)
    centres = rng.uniform(0.8 * s0, 1.2 * s0, 500)
    sig = 0.05 * s0
    v = 1.2 * np.exp(-(s - centres) ** 2 / (2 * sig * sig))
    return v.sum(), (v * (-(s - centres) / (sig * sig))).sum()


def make(line, prec):
    from plumed2_gb300.action import Coordination
    return Coordination(line, precision=prec)


CASES = [
    ("GROUPA=1-216 SWITCH={RATIONAL R_0=0.3 NN=6 MM=12 D_MAX=0.9}", "SWITCH={RATIONAL R_0=%r NN=6 MM=12 D_MAX=0.9 D_0=%r}"),
    ("GROUPA=1-216 R_0=0.3", "R_0=%r D_0=%r"),
    ("GROUPA=1-108 GROUPB=109-216 SWITCH={RATIONAL R_0=0.3 NN=6 MM=12 D_MAX=0.9} NLIST NL_CUTOFF=1.0 NL_STRIDE=5",
     "SWITCH={RATIONAL R_0=%r NN=6 MM=12 D_MAX=0.9 D_0=%r} NLIST NL_CUTOFF=1.0 NL_STRIDE=5"),
]


@pytest.mark.parametrize("line,pline", CASES)
def test_backward_fp64_against_oracle_and_fd(orc, line, pline):
    from plumed2_gb300.autograd import coordination
    dev = torch.device("cuda:0")
    pos0 = jittered_lattice(216, 0.3, 0.04, 11)
    L = 1.8
    box0 = np.diag([L, L, L])
    act = make(line, "fp64")
    pos = torch.tensor(pos0[None], dtype=torch.float64, device=dev, requires_grad=True)
    box = torch.tensor(box0, dtype=torch.float64, requires_grad=True)
    r0 = torch.tensor(0.3, dtype=torch.float64, device=dev, requires_grad=True)
    d0 = torch.tensor(0.0, dtype=torch.float64, device=dev, requires_grad=True)
    s = coordination(act, pos, box, r0, d0)
    s0 = float(s.item())
    V = bias(s, s0).sum()
    V.backward()
    gpos = pos.grad[0].cpu().numpy()
    gbox = box.grad.numpy()
    # oracle analytic derivatives x V'(s)
    is_nl = "NLIST" in line
    if "GROUPB" in line:
        pairs = orc.nl_classic(1, 108, 108, pos0, box0, True, 1.0) if is_nl else orc.all_pairs(1, 108, 108)
    else:
        pairs = orc.all_pairs(0, 216)
    spec = "RATIONAL R_0=0.3 NN=6 MM=12 D_MAX=0.9" if "SWITCH" in line else "R0SYNTAX 6 0 0.3 0.0"
    so, do, vo = orc.coordination(spec, pos0, box0, pairs)
    _, dV = bias_np(so, s0)
    assert abs(so - s0) <= 1e-12 * abs(so)
    assert np.abs(gpos - dV * do).max() <= 1e-10 * np.abs(dV * do).max()
    ref_box = dV * (-np.linalg.inv(box0).T @ vo)
    assert np.abs(gbox - ref_box).max() <= 1e-10 * np.abs(ref_box).max()

    # central finite differences of V in FP64 (fresh actions, same NL where used)
    def V_of(p, b, r0v=0.3, d0v=0.0):
        a = make(line.split(" SWITCH")[0].split(" R_0")[0] + " " + (pline % (r0v, d0v)), "fp64")
        sv, _, _ = a.calculate(p, b, 0, derivatives=False)
        a.close()
        return bias_np(sv, s0)[0]

    h = 1e-6
    rng = np.random.default_rng(0)
    for idx in rng.choice(216, 4, replace=False):
        for k in range(3):
            pp = pos0.copy()
            pm = pos0.copy()
            pp[idx, k] += h
            pm[idx, k] -= h
            fd = (V_of(pp, box0) - V_of(pm, box0)) / (2 * h)
            assert abs(fd - gpos[idx, k]) <= 2e-6 * np.abs(gpos).max() + 1e-9, (idx, k, fd, gpos[idx, k])
    scaled = pos0 @ np.linalg.inv(box0)
    for (kk, bb) in ((0, 0), (1, 1), (2, 2), (0, 1)):
        bp = box0.copy()
        bm = box0.copy()
        bp[kk, bb] += h
        bm[kk, bb] -= h
        fd = (V_of(scaled @ bp, bp) - V_of(scaled @ bm, bm)) / (2 * h)
        assert abs(fd - gbox[kk, bb]) <= 2e-6 * np.abs(gbox).max() + 1e-9, (kk, bb, fd, gbox[kk, bb])
    fd_r0 = (V_of(pos0, box0, 0.3 + h) - V_of(pos0, box0, 0.3 - h)) / (2 * h)
    assert abs(fd_r0 - r0.grad.item()) <= 2e-6 * abs(fd_r0) + 1e-9, (fd_r0, r0.grad.item())
    fd_d0 = (V_of(pos0, box0, 0.3, h) - V_of(pos0, box0, 0.3, -h)) / (2 * h)
    assert abs(fd_d0 - d0.grad.item()) <= 2e-6 * abs(fd_d0) + 1e-9, (fd_d0, d0.grad.item())
    act.close()


def test_backward_mixed_matches_fp64():
    from plumed2_gb300.autograd import coordination
    dev = torch.device("cuda:0")
    n, L = 4096, 16 * 0.31
    line = "GROUPA=1-%d SWITCH={RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.6} NLIST NL_CUTOFF=0.8 NL_STRIDE=10" % n
    frames = np.stack([jittered_lattice(n, 0.31, 0.03, 40 + w) for w in range(2)])
    out = {}
    for prec in ("fp64", "mixed"):
        act = make(line, prec)
        pos = torch.tensor(frames, dtype=torch.float64, device=dev, requires_grad=True)
        box = torch.tensor(np.diag([L] * 3), dtype=torch.float64, requires_grad=True)
        r0 = torch.tensor(0.32, dtype=torch.float64, device=dev, requires_grad=True)
        d0 = torch.tensor(0.0, dtype=torch.float64, device=dev, requires_grad=True)
        s = coordination(act, pos, box, r0, d0)
        s0 = float(s[0].item()) if prec == "fp64" else out["fp64"][0][0]
        V = bias(s, s0).sum()
        V.backward()
        out[prec] = (s.detach().cpu().numpy(), pos.grad.cpu().numpy(), box.grad.numpy(), r0.grad.item(),
                     d0.grad.item())
        act.close()
    a, b = out["fp64"], out["mixed"]
    assert np.all(np.abs(a[0] - b[0]) <= 1e-6 * np.abs(a[0]))
    assert np.abs(a[1] - b[1]).max() <= 1e-5 * np.abs(a[1]).max()
    assert np.abs(a[2] - b[2]).max() <= 1e-5 * np.abs(a[2]).max()
    assert abs(a[3] - b[3]) <= 1e-5 * abs(a[3])
    assert abs(a[4] - b[4]) <= 1e-5 * abs(a[4])


def test_forward_dr0_flag_matches_backward():
    """COORD_FLAG_DR0 on the forward returns ds/dR_0, ds/dD_0 (g = 1)."""
    from plumed2_gb300 import _lib
    dev = torch.device("cuda:0")
    act = make("GROUPA=1-512 SWITCH={RATIONAL R_0=0.3 NN=6 MM=12 D_MAX=0.9}", "fp64")
    pos = torch.tensor(jittered_lattice(512, 0.3, 0.04, 12)[None], dtype=torch.float64, device=dev)
    box = np.diag([2.4] * 3)[None]
    s = torch.zeros(1, dtype=torch.float64, device=dev)
    der = torch.zeros(1, 512, 3, dtype=torch.float64, device=dev)
    vir = torch.zeros(1, 9, dtype=torch.float64, device=dev)
    dp = torch.zeros(1, 2, dtype=torch.float64, device=dev)
    act.forward_device(pos.data_ptr(), box, 1, s.data_ptr(), der.data_ptr(), vir.data_ptr(), flags=_lib.FLAG_DR0,
                       dparam_ptr=dp.data_ptr())
    g = torch.ones(1, dtype=torch.float64, device=dev)
    gp = torch.zeros_like(der)
    gb = torch.zeros(1, 9, dtype=torch.float64, device=dev)
    gq = torch.zeros(1, 2, dtype=torch.float64, device=dev)
    act.backward_device(pos.data_ptr(), box, 1, g.data_ptr(), gp.data_ptr(), gb.data_ptr(), gq.data_ptr())
    torch.cuda.synchronize()
    assert torch.allclose(gp, der, rtol=1e-12, atol=1e-14)
    assert torch.allclose(gq, dp, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_saved_forward_matches_recompute(prec):
    """COORD_FLAG_SAVE keeps ds/dx and the virial of the forward (and
    ds/d(R_0, D_0) with COORD_FLAG_DR0); the next backward scales them instead
    of re-running the pairs.  Every route gives the same gradients (1e-12
    relative on FP64, 1e-6 mixed: only the order of the atomic additions
    differs) and a SAVE forward still hands back its own derivatives."""
    from plumed2_gb300 import _lib
    dev = torch.device("cuda:0")
    n, L, F = 1000, 10 * 0.31, 2
    line = "GROUPA=1-%d SWITCH={RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.9} NLIST NL_CUTOFF=1.0 NL_STRIDE=10" % n
    frames = np.stack([jittered_lattice(n, 0.31, 0.03, 60 + f) for f in range(F)])
    boxes = np.stack([np.diag([L] * 3)] * F)
    pos = torch.tensor(frames, dtype=torch.float64, device=dev)
    g = torch.tensor([0.7, -1.3], dtype=torch.float64, device=dev)
    routes = {"recompute": (0, True), "save": (_lib.FLAG_SAVE, False), "save+dr0": (_lib.FLAG_SAVE | _lib.FLAG_DR0, True),
              "save, params recomputed": (_lib.FLAG_SAVE, True)}
    res = {}
    for name, (flags, want_param) in routes.items():
        act = make(line, prec)
        s = torch.zeros(F, dtype=torch.float64, device=dev)
        der = torch.zeros(F, n, 3, dtype=torch.float64, device=dev)
        vir = torch.zeros(F, 9, dtype=torch.float64, device=dev)
        dp = torch.zeros(F, 2, dtype=torch.float64, device=dev)
        act.forward_device(pos.data_ptr(), boxes, F, s.data_ptr(), der.data_ptr(), vir.data_ptr(), step=0,
                           flags=flags, dparam_ptr=dp.data_ptr() if flags & _lib.FLAG_DR0 else 0)
        gp = torch.zeros(F, n, 3, dtype=torch.float64, device=dev)
        gb = torch.zeros(F, 9, dtype=torch.float64, device=dev)
        gq = torch.zeros(F, 2, dtype=torch.float64, device=dev)
        act.backward_device(pos.data_ptr(), boxes, F, g.data_ptr(), gp.data_ptr(), gb.data_ptr(),
                            gq.data_ptr() if want_param else 0)
        torch.cuda.synchronize()
        res[name] = [t.cpu().numpy() for t in (s, der, vir, gp, gb, gq)]
        if flags & _lib.FLAG_DR0:
            assert np.abs(dp.cpu().numpy() * g.cpu().numpy()[:, None] - res[name][5]).max() <= \
                1e-14 * np.abs(res[name][5]).max()
        act.close()
    tol = 1e-12 if prec == "fp64" else 1e-6
    ref = res["recompute"]
    for name, got in res.items():
        for k, (a, b) in enumerate(zip(ref, got)):
            if k == 5 and not routes[name][1]:
                assert np.all(b == 0.0)  # no grad_param requested
                continue
            assert np.abs(a - b).max() <= tol * max(np.abs(a).max(), 1e-300), (name, k)
        # the saved gradient is g times the forward's own derivatives: exactly
        # on FP64; the mixed path forms the product in FP32 (its derivatives
        # are FP32-accurate), within 2^-23 relative of each component
        if name in ("save", "save+dr0"):
            s_, der, vir, gp = got[:4]
            want = g.cpu().numpy()[:, None, None] * der
            if prec == "fp64":
                assert np.abs(gp - want).max() <= 1e-14 * np.abs(gp).max()
            else:
                assert np.all(np.abs(gp - want) <= 2.0 ** -23 * np.abs(want))


def test_c3_metad_backward_at_size(orc):
    """The differentiation workload at its own size: the 32,768-atom two-slab
    system (GROUPA = the z < L/2 slab, GROUPB = the other, RATIONAL R_0=0.35
    D_MAX=1.2, NLIST NL_CUTOFF=1.4), s feeding 500 hills (h = 1.2, sigma =
    0.05 s0, centres uniform in [0.8 s0, 1.2 s0], s0 = frame 0's CV).
    FP64: dV/dx and dV/dh against the oracle's analytic derivatives times
    V'(s) (1e-10 of their scale), and against FP64 central differences with
    h = 1e-6 nm for eight sampled atoms (all three coordinates), four box
    entries (scaled coordinates fixed), R_0 and D_0 (2e-6 of the gradient's
    scale).  Mixed: the same gradients within 1e-5 of the FP64 ones."""
    from plumed2_gb300 import frames as W
    from plumed2_gb300.autograd import coordination
    dev = torch.device("cuda:0")
    frames, box0 = W.workload_c1(n_frames=1)
    pos0 = frames[0]
    n, half = len(pos0), len(pos0) // 2
    pline = ("GROUPA=1-%d GROUPB=%d-%d SWITCH={RATIONAL R_0=%%r NN=6 MM=12 D_MAX=1.2 D_0=%%r} NLIST NL_CUTOFF=1.4 "
             "NL_STRIDE=20" % (half, half + 1, n))
    line = pline % (0.35, 0.0)
    out = {}
    for prec in ("fp64", "mixed"):
        act = make(line, prec)
        pos = torch.tensor(pos0[None], dtype=torch.float64, device=dev, requires_grad=True)
        box = torch.tensor(box0, dtype=torch.float64, requires_grad=True)
        r0 = torch.tensor(0.35, dtype=torch.float64, device=dev, requires_grad=True)
        d0 = torch.tensor(0.0, dtype=torch.float64, device=dev, requires_grad=True)
        s = coordination(act, pos, box, r0, d0)
        s0 = float(s.item()) if prec == "fp64" else out["fp64"][0]
        V = bias(s, s0).sum()
        V.backward()
        out[prec] = (s0 if prec == "fp64" else float(s.item()), pos.grad[0].cpu().numpy(), box.grad.numpy(),
                     r0.grad.item(), d0.grad.item())
        act.close()
    s0, gpos, gbox, gr0, gd0 = out["fp64"]
    # the oracle's analytic derivatives (the reference's layout) times V'(s)
    pairs = orc.nl_classic_cells(1, half, half, pos0, box0, True, 1.4)
    so, do, vo = orc.coordination("RATIONAL R_0=0.35 NN=6 MM=12 D_MAX=1.2", pos0, box0, pairs,
                                  nthreads=orc.max_threads())
    assert abs(so - s0) <= 1e-12 * abs(so)
    _, dV = bias_np(so, s0)
    assert np.abs(gpos - dV * do).max() <= 1e-10 * np.abs(dV * do).max()
    ref_box = dV * (-np.linalg.inv(box0).T @ vo)
    assert np.abs(gbox - ref_box).max() <= 1e-10 * np.abs(ref_box).max()

    def V_of(p, b, r0v=0.35, d0v=0.0):
        a = make(pline % (r0v, d0v), "fp64")
        sv, _, _ = a.calculate(p, b, 0, derivatives=False)
        a.close()
        return bias_np(sv, s0)[0]

    h = 1e-6
    rng = np.random.default_rng(5)
    # sampled atoms: four near the slab interfaces (non-zero forces), four anywhere
    near = np.flatnonzero(np.linalg.norm(gpos, axis=1) > 0.1 * np.linalg.norm(gpos, axis=1).max())
    idxs = list(rng.choice(near, 4, replace=False)) + list(rng.choice(n, 4, replace=False))
    gscale = np.abs(gpos).max()
    for idx in idxs:
        for k in range(3):
            pp = pos0.copy()
            pm = pos0.copy()
            pp[idx, k] += h
            pm[idx, k] -= h
            fd = (V_of(pp, box0) - V_of(pm, box0)) / (2 * h)
            assert abs(fd - gpos[idx, k]) <= 2e-6 * gscale + 1e-9, (idx, k, fd, gpos[idx, k])
    scaled = pos0 @ np.linalg.inv(box0)
    for (kk, bb) in ((0, 0), (1, 1), (2, 2), (0, 2)):
        bp = box0.copy()
        bm = box0.copy()
        bp[kk, bb] += h
        bm[kk, bb] -= h
        fd = (V_of(scaled @ bp, bp) - V_of(scaled @ bm, bm)) / (2 * h)
        assert abs(fd - gbox[kk, bb]) <= 2e-6 * np.abs(gbox).max() + 1e-9, (kk, bb, fd, gbox[kk, bb])
    fd_r0 = (V_of(pos0, box0, 0.35 + h) - V_of(pos0, box0, 0.35 - h)) / (2 * h)
    assert abs(fd_r0 - gr0) <= 2e-6 * abs(fd_r0) + 1e-9, (fd_r0, gr0)
    fd_d0 = (V_of(pos0, box0, 0.35, h) - V_of(pos0, box0, 0.35, -h)) / (2 * h)
    assert abs(fd_d0 - gd0) <= 2e-6 * abs(fd_d0) + 1e-9, (fd_d0, gd0)
    # mixed precision against FP64
    sm, gpm, gbm, gr0m, gd0m = out["mixed"]
    assert abs(sm - s0) <= 1e-6 * abs(s0)
    assert np.sqrt(((gpm - gpos) ** 2).sum(axis=1)).max() <= 1e-5 * np.sqrt((gpos ** 2).sum(axis=1)).max()
    assert np.abs(gbm - gbox).max() <= 1e-5 * np.abs(gbox).max()
    assert abs(gr0m - gr0) <= 1e-5 * abs(gr0)
    assert abs(gd0m - gd0) <= 1e-5 * abs(gd0)
