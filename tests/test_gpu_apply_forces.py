"""Force application on the device (coord_apply_forces) after a saved forward:
atom_forces[f][abs(i)] += ff[f] * ds/dx_i and box_forces[f] += ff[f] * virial[f]
(Colvar::apply with ActionWithValue::checkForForces and
ActionAtomistic::setForcesOnAtoms / setForcesOnCell), against the same sums
formed in numpy from the forward's own derivatives and virial.  An atom in
both groups receives both of its slots' forces.  Tolerance 1e-12 relative
(only the order of additions differs)."""
import numpy as np
import pytest

from plumed2_gb300.frames import jittered_lattice

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("groups,nlist", [("GROUPA=101-900 GROUPB=501-1400", True),
                                          ("GROUPA=1-3000", True), ("GROUPA=11-610", False)])
def test_apply_forces_matches_scatter(prec, groups, nlist):
    from plumed2_gb300 import _lib
    from plumed2_gb300.action import Coordination
    dev = torch.device("cuda:0")
    n_sys, L, F = 3375, 15 * 0.31, 2
    frames = np.stack([jittered_lattice(n_sys, 0.31, 0.03, 90 + f) for f in range(F)])
    boxes = np.stack([np.diag([L] * 3)] * F)
    line = "%s SWITCH={RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.9}" % groups
    if nlist:
        line += " NLIST NL_CUTOFF=1.0 NL_STRIDE=10"
    c = Coordination(line, precision=prec)
    idx = np.asarray(c.requested_atoms)
    pos = torch.tensor(frames[:, idx], dtype=torch.float64, device=dev).contiguous()
    ns = len(idx)
    s = torch.zeros(F, dtype=torch.float64, device=dev)
    der = torch.zeros(F, ns, 3, dtype=torch.float64, device=dev)
    vir = torch.zeros(F, 9, dtype=torch.float64, device=dev)
    with pytest.raises(_lib.CoordError):  # nothing saved yet
        c.apply_forces(F, s.data_ptr(), n_sys)
    c.forward_device(pos.data_ptr(), boxes, F, s.data_ptr(), der.data_ptr(), vir.data_ptr(), step=0,
                     flags=_lib.FLAG_SAVE)
    rng = np.random.default_rng(1)
    f0 = rng.normal(size=(F, n_sys, 3))
    b0 = rng.normal(size=(F, 9))
    forces = torch.tensor(f0, dtype=torch.float64, device=dev)
    box_f = torch.tensor(b0, dtype=torch.float64, device=dev)
    ff = torch.tensor([-1.7, 0.4], dtype=torch.float64, device=dev)
    c.apply_forces(F, ff.data_ptr(), n_sys, forces.data_ptr(), box_f.data_ptr())
    torch.cuda.synchronize()
    D, V = der.cpu().numpy(), vir.cpu().numpy()
    exp_f = f0.copy()
    for f in range(F):
        np.add.at(exp_f[f], idx, ff[f].item() * D[f])
    exp_b = b0 + ff.cpu().numpy()[:, None] * V
    got = forces.cpu().numpy()
    scale = np.abs(exp_f - f0).max()
    assert np.abs(got - exp_f).max() <= 1e-12 * scale + 1e-15
    np.testing.assert_allclose(box_f.cpu().numpy(), exp_b, rtol=1e-13, atol=1e-13)
    with pytest.raises(_lib.CoordError):  # the saved state is consumed
        c.apply_forces(F, ff.data_ptr(), n_sys, forces.data_ptr())
    c.close()
