"""Device biases on the CV (coord_bias_hills, coord_bias_restraint) against a
numpy restatement of the reference's formulas:

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

DP2CUT = 6.25


def hills_ref(s, c, sg, h, stretch):
    a = 1.0 / (1.0 - np.exp(-DP2CUT)) if stretch else 1.0
    b = -np.exp(-DP2CUT) / (1.0 - np.exp(-DP2CUT)) if stretch else 0.0
    dp = (s[:, None] - c) / sg
    dp2 = 0.5 * dp * dp
    on = dp2 < DP2CUT
    e = np.where(on, h * np.exp(-dp2), 0.0)
    V = (a * e + np.where(on, h * b, 0.0)).sum(1)
    dV = (-a * e * dp / sg).sum(1)
    return V, dV


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
    V0, dV0 = hills_ref(s, c, sg, h, stretch)
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
    cv = s - 0.7
    np.testing.assert_allclose(V.cpu().numpy(), 2.0 + 0.5 * 3.5 * cv * cv - 0.25 * cv, rtol=1e-14)
    np.testing.assert_allclose(dV.cpu().numpy(), -1.0 + 3.5 * cv - 0.25, rtol=1e-14, atol=1e-14)


def test_bias_argument_errors():
    from plumed2_gb300 import _lib
    with pytest.raises(_lib.CoordError):
        _lib.bias_hills(2, 0, 3, 0, 0, 0)
    with pytest.raises(_lib.CoordError):
        _lib.bias_restraint(2, 0, 0.0, 1.0)
