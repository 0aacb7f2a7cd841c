"""Device biases on the CV (coord_bias_hills, coord_bias_restraint) against the
reference's own METAD and RESTRAINT outputs (regtest goldens, at the end) and a
numpy restatement of the reference's formulas (oracle.metad_hills,
oracle.restraint):

* hills: MetaD::evaluateGaussianAndDerivatives, non-multivariate branch
  (src/bias/MetaD.cpp:2256-2273): dp = (s - c)/sigma, dp2 = dp^2/2; for
  dp2 < 6.25 the hill adds h*(A*exp(-dp2) + B) to V and -A*h*exp(-dp2)*dp/sigma
  to dV/ds, with A, B the stretch constants of src/tools/Tools.h:71-74;
* restraint: Restraint::calculate (src/bias/Restraint.cpp:125-141).
Tolerance: 1e-13 relative (FP64; only the summation order differs).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("stretch", [True, False])
@pytest.mark.parametrize("n_hills", [0, 1, 7, 500, 4099])
def test_hills_match_restatement(stretch, n_hills):
    from plumed2_gb300 import _lib
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(n_hills + 17)
    F = 5
    s = rng.uniform(100.0, 200.0, F)
    c = rng.uniform(80.0, 220.0, (F, n_hills))
    sg = rng.uniform(2.0, 12.0, (F, n_hills))
    h = rng.uniform(0.1, 1.5, (F, n_hills))
    ts, tc, tsg, th = (torch.tensor(x, dtype=torch.float64, device=dev).contiguous() for x in (s, c, sg, h))
    V = torch.zeros(F, dtype=torch.float64, device=dev)
    dV = torch.zeros(F, dtype=torch.float64, device=dev)
    _lib.bias_hills(F, ts.data_ptr(), n_hills, tc.data_ptr(), tsg.data_ptr(), th.data_ptr(), V.data_ptr(),
                    dV.data_ptr(), stretch=stretch)
    torch.cuda.synchronize()
    from oracle import metad_hills
    V0, dV0 = metad_hills(s, c, sg, h, stretch)
    np.testing.assert_allclose(V.cpu().numpy(), V0, rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(dV.cpu().numpy(), dV0, rtol=1e-12, atol=1e-14 * (np.abs(dV0).max() + 1e-300))


def test_restraint_and_accumulate():
    from plumed2_gb300 import _lib
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(3)
    F = 300
    s = rng.uniform(-5, 5, F)
    ts = torch.tensor(s, dtype=torch.float64, device=dev)
    V = torch.full((F,), 2.0, dtype=torch.float64, device=dev)
    dV = torch.full((F,), -1.0, dtype=torch.float64, device=dev)
    _lib.bias_restraint(F, ts.data_ptr(), 0.7, 3.5, -0.25, V.data_ptr(), dV.data_ptr(), accumulate=True)
    torch.cuda.synchronize()
    from oracle import restraint
    V0, dV0 = restraint(s, 0.7, 3.5, -0.25)
    np.testing.assert_allclose(V.cpu().numpy(), 2.0 + V0, rtol=1e-14)
    np.testing.assert_allclose(dV.cpu().numpy(), -1.0 + dV0, rtol=1e-14, atol=1e-14)


def test_bias_argument_errors():
    from plumed2_gb300 import _lib
    with pytest.raises(_lib.CoordError):
        _lib.bias_hills(2, 0, 3, 0, 0, 0)
    with pytest.raises(_lib.CoordError):
        _lib.bias_restraint(2, 0, 0.0, 1.0)


def test_hills_reproduce_reference_metad_forces(orc, golden):
    """regtest/basic/rt-metad-numder: METAD (SIGMA=0.1, HEIGHT=1.0, PACE=10,
    stretched Gaussians) on d1 = DISTANCE ATOMS=1,10 over five frames of
    regtest/trajectories/trajectory.xyz (stride 10).  No hill on the first
    step (MetaD::update, src/bias/MetaD.cpp:2377-2385); frame k feels the
    hills deposited at d1 of the frames before it.  coord_bias_hills gives
    dV/dd1 on the device; -dV/dd1 * dd1/dx reproduces the reference's
    analytical forces on atoms 1 and 10 (%8.4f)."""
    from plumed2_gb300 import _lib
    g = golden("rt_metad_numder.json")
    dev = torch.device("cuda:0")
    d, u = [], []
    for fr, bx in zip(g["frames"], g["box"]):
        v = orc.pbc_distance(np.diag(bx), np.array(fr[0]), np.array(fr[1]))[0]
        d.append(float(np.sqrt(v @ v)))
        u.append(v / d[-1])
    deposit = [k for k in range(len(d)) if (k * g["trajectory_stride"]) % g["pace"] == 0 and k > 0]
    for k in range(len(d)):
        seen = [d[j] for j in deposit if j < k]
        n = len(seen)
        ts = torch.tensor([d[k]], dtype=torch.float64, device=dev)
        tc = torch.tensor([seen], dtype=torch.float64, device=dev).reshape(1, n)
        tsg = torch.full((1, n), g["sigma"], dtype=torch.float64, device=dev)
        th = torch.full((1, n), g["height"], dtype=torch.float64, device=dev)
        V = torch.zeros(1, dtype=torch.float64, device=dev)
        dV = torch.zeros(1, dtype=torch.float64, device=dev)
        _lib.bias_hills(1, ts.data_ptr(), n, tc.data_ptr(), tsg.data_ptr(), th.data_ptr(), V.data_ptr(),
                        dV.data_ptr(), stretch=True)
        torch.cuda.synchronize()
        f10 = -dV.item() * u[k]
        assert np.abs(f10 - np.array(g["forces_atom10"][k])).max() <= 5.01e-5, (k, f10, g["forces_atom10"][k])
        assert np.abs(-f10 - np.array(g["forces_atom1"][k])).max() <= 5.01e-5, k


def test_restraint_forces_reproduce_rt_mpi0(golden):
    """regtest/basic/rt-mpi0: RESTRAINT ARG=c KAPPA=5 AT=15 on COORDINATION
    GROUPA=1-10 GROUPB=30-40,5,50-100.  On the device: the FP64 forward with
    its derivatives kept (COORD_FLAG_SAVE), the restraint's dV/ds
    (coord_bias_restraint), then the forces -dV/ds * ds/dx scattered by atom
    number and the box force (coord_apply_forces).  They reproduce the
    reference's forces and virial diagonal (ff.0.reference, %f)."""
    from plumed2_gb300 import _lib
    from plumed2_gb300.action import Coordination
    g = golden("rt_mpi0.json")
    rs = g["restraint"]
    c = Coordination("GROUPA=%s GROUPB=%s SWITCH={%s}" % (g["groupa"], g["groupb"], g["switch"][rs["arg"]]),
                     precision="fp64")
    idx = np.asarray(c.requested_atoms)
    dev = torch.device("cuda:0")
    for fi, (fr, bx) in enumerate(zip(g["frames"], g["box"])):
        frame = np.array(fr)
        box = np.diag(bx) if len(bx) == 3 else np.array(bx).reshape(3, 3)
        pos = torch.tensor(frame[idx][None], dtype=torch.float64, device=dev).contiguous()
        s = torch.zeros(1, dtype=torch.float64, device=dev)
        c.forward_device(pos.data_ptr(), box[None], 1, s.data_ptr(), 0, 0, step=fi, flags=_lib.FLAG_SAVE)
        V = torch.zeros(1, dtype=torch.float64, device=dev)
        dV = torch.zeros(1, dtype=torch.float64, device=dev)
        _lib.bias_restraint(1, s.data_ptr(), rs["at"], rs["kappa"], 0.0, V.data_ptr(), dV.data_ptr())
        ff = -dV
        forces = torch.zeros(1, len(frame), 3, dtype=torch.float64, device=dev)
        boxf = torch.zeros(1, 9, dtype=torch.float64, device=dev)
        c.apply_forces(1, ff.data_ptr(), len(frame), forces.data_ptr(), boxf.data_ptr())
        torch.cuda.synchronize()
        assert np.abs(forces[0].cpu().numpy() - np.array(g["ff_forces"][fi])).max() <= 5.01e-7, fi
        vd = boxf[0].cpu().numpy().reshape(3, 3).diagonal()
        assert np.abs(vd - np.array(g["ff_virial_diag"][fi])).max() <= 5.01e-7, fi
    c.close()
