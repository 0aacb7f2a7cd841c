"""The host-buffer call (coord_forward) moves data two ways: kernels that
access the caller's pageable arrays in place (devices that use the host page
tables, e.g. behind NVLink-C2C), or copies staged through pinned buffers
(COORD_HOST_STAGED=1, and every other device).  Both give the same results as
the device-pointer call on the same inputs (FP64 path: 1e-12 relative; only
the order of the atomic additions differs)."""
import os

import numpy as np
import pytest

from plumed2_gb300.frames import jittered_lattice

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("nlist", [True, False])
def test_direct_and_staged_host_paths_agree(prec, nlist):
    """Step 0 rebuilds the list (positions copied to the device); step 1 does
    not (mixed path: positions and derivatives move in one pass each)."""
    from plumed2_gb300.action import Coordination
    n, L = 2000, 13 * 0.31
    line = "GROUPA=1-%d SWITCH={RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.9}" % n
    if nlist:
        line += " NLIST NL_CUTOFF=1.0 NL_STRIDE=10"
    pos = jittered_lattice(n, 0.31, 0.03, 70)
    box = np.diag([L] * 3)
    res = {}
    for staged in (False, True):
        if staged:
            os.environ["COORD_HOST_STAGED"] = "1"
        try:
            c = Coordination(line, precision=prec)
            out = (np.zeros((n, 3)), np.zeros(9))
            r0 = c.calculate(pos, box, 0)
            r1 = c.calculate(pos, box, 1, out=out)
            assert r1[1] is out[0]
            res[staged] = (r0, r1)
            c.close()
        finally:
            os.environ.pop("COORD_HOST_STAGED", None)
    # the device-pointer call on the same inputs
    c = Coordination(line, precision=prec)
    dev = torch.device("cuda:0")
    tp = torch.tensor(pos[None], dtype=torch.float64, device=dev)
    s = torch.zeros(1, dtype=torch.float64, device=dev)
    d = torch.zeros(1, n, 3, dtype=torch.float64, device=dev)
    v = torch.zeros(1, 9, dtype=torch.float64, device=dev)
    c.forward_device(tp.data_ptr(), box[None], 1, s.data_ptr(), d.data_ptr(), v.data_ptr(), step=0)
    torch.cuda.synchronize()
    ref = (s.item(), d[0].cpu().numpy(), v[0].cpu().numpy().reshape(3, 3))
    c.close()
    tol = 1e-12 if prec == "fp64" else 1e-6
    for staged in (False, True):
        for got in res[staged]:
            assert abs(got[0] - ref[0]) <= tol * abs(ref[0])
            assert np.abs(got[1] - ref[1]).max() <= tol * np.abs(ref[1]).max()
            assert np.abs(got[2] - ref[2]).max() <= tol * np.abs(ref[2]).max()


def test_self_pair_only_host_call():
    from plumed2_gb300.action import Coordination
    c = Coordination("GROUPA=1 GROUPB=1 R_0=0.3")
    s, d, v = c.calculate(np.zeros((2, 3)), np.diag([3.0] * 3))
    assert s == 0.0 and np.all(d == 0) and np.all(v == 0)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("path", ["direct", "staged", "pinned"])
def test_batched_host_call_equals_device_call(prec, path):
    """coord_forward_batch: three walkers' host arrays in one call, on a
    rebuild step and on a plain step, equal the batched device call
    (pinned: page-locked arrays, moved chunk by chunk on the copy engines on
    the mixed path)."""
    from plumed2_gb300.action import Coordination
    from plumed2_gb300._lib import addr
    n, F, L = 2000, 3, 13 * 0.31
    line = "GROUPA=1-%d SWITCH={RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.9} NLIST NL_CUTOFF=1.0 NL_STRIDE=10" % n
    if path == "pinned":
        arr = lambda *shape: torch.zeros(*shape, dtype=torch.float64, pin_memory=True).numpy()
    else:
        arr = lambda *shape: np.zeros(shape)
    pos = arr(F, n, 3)
    pos[:] = np.stack([jittered_lattice(n, 0.31, 0.03, 80 + f) for f in range(F)])
    boxes = np.ascontiguousarray(np.stack([np.diag([L] * 3).reshape(9)] * F))
    if path == "staged":
        os.environ["COORD_HOST_STAGED"] = "1"
    try:
        c = Coordination(line, precision=prec)
        got = []
        for step in (0, 1, 2):
            s, d, v = arr(F), arr(F, n, 3), arr(F, 9)
            c.forward_host_batch(F, addr(pos), addr(boxes), step, 0, addr(s), addr(d), addr(v))
            got.append((s.copy(), d.copy(), v.copy()))
        c.close()
    finally:
        os.environ.pop("COORD_HOST_STAGED", None)
    c = Coordination(line, precision=prec)
    dev = torch.device("cuda:0")
    tp = torch.tensor(pos, dtype=torch.float64, device=dev)
    s = torch.zeros(F, dtype=torch.float64, device=dev)
    d = torch.zeros(F, n, 3, dtype=torch.float64, device=dev)
    v = torch.zeros(F, 9, dtype=torch.float64, device=dev)
    c.forward_device(tp.data_ptr(), boxes, F, s.data_ptr(), d.data_ptr(), v.data_ptr(), step=0)
    torch.cuda.synchronize()
    ref = (s.cpu().numpy(), d.cpu().numpy(), v.cpu().numpy())
    c.close()
    tol = 1e-12 if prec == "fp64" else 1e-6
    for g in got:
        for f in range(F):
            assert abs(g[0][f] - ref[0][f]) <= tol * abs(ref[0][f])
            assert np.abs(g[1][f] - ref[1][f]).max() <= tol * np.abs(ref[1][f]).max()
            assert np.abs(g[2][f] - ref[2][f]).max() <= tol * np.abs(ref[2][f]).max()


def test_pinned_batch_skin_follows_every_walker():
    """The pinned batched call moves its walkers in chunks; the displacements
    each chunk measures go to its own walkers' slots, so the skin chosen at a
    rebuild (from the largest displacement of the interval over every walker)
    is the device call's on the same trajectory, and so are the near parts."""
    from plumed2_gb300.action import Coordination
    from plumed2_gb300._lib import addr
    n, F, L = 2744, 8, 14 * 0.31
    line = "GROUPA=1-%d SWITCH={RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.6} NLIST NL_CUTOFF=0.8 NL_STRIDE=10" % n
    pin = lambda *shape: torch.zeros(*shape, dtype=torch.float64, pin_memory=True).numpy()
    rng = np.random.default_rng(4)
    traj = [np.stack([jittered_lattice(n, 0.31, 0.03, 90 + f) for f in range(F)])]
    for k in range(1, 21):
        # walker f moves with its own step size: the largest moves are the first chunk's
        traj.append(traj[-1] + rng.normal(0.0, 1.0, (F, n, 3)) * (0.0003 * (F - np.arange(F)))[:, None, None])
    boxes = np.ascontiguousarray(np.stack([np.diag([L] * 3).reshape(9)] * F))
    ch = Coordination(line, precision="mixed")
    pos, s, d, v = pin(F, n, 3), pin(F), pin(F, n, 3), pin(F, 9)
    dev = torch.device("cuda:0")
    cd = Coordination(line, precision="mixed")
    sd = torch.zeros(F, dtype=torch.float64, device=dev)
    dd = torch.zeros(F, n, 3, dtype=torch.float64, device=dev)
    vd = torch.zeros(F, 9, dtype=torch.float64, device=dev)
    from plumed2_gb300 import _lib
    pageable, tables = _lib.host_memory_access(0)
    direct = bool(pageable and tables) and os.environ.get("COORD_HOST_STAGED") != "1"
    for step in range(21):
        pos[:] = traj[step]
        ch.forward_host_batch(F, addr(pos), addr(boxes), step, 0, addr(s), addr(d), addr(v))
        # the path the call reports: copy-engine chunks between rebuilds, the
        # kernels' direct access on a rebuild step (or staging without access)
        assert ch.host_path() == (("direct" if step % 10 == 0 else "chunked") if direct else "staged"), step
        tp = torch.tensor(traj[step], dtype=torch.float64, device=dev)
        cd.forward_device(tp.data_ptr(), boxes, F, sd.data_ptr(), dd.data_ptr(), vd.data_ptr(), step=step)
        torch.cuda.synchronize()
        for f in range(F):
            assert abs(s[f] - sd[f].item()) <= 1e-6 * abs(sd[f].item()), (step, f)
    for f in range(F):
        assert ch.nl_near_size(f) == cd.nl_near_size(f), f
    ch.close()
    cd.close()
