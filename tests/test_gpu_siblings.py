"""DHENERGY and GHBFIX (CoordinationBase's loop with their own pairing()) on
the GPU, through the C ABI, against the reference's regtest goldens and the
FP64 oracle on the same inputs.

Tolerances:
  goldens      the print format of the reference file (%6.5f, %8.4f)
  oracle       s: |ds| <= 1e-12 * sum_pairs |term| (DHENERGY sums terms of
               both signs, so the scale is the sum of their magnitudes);
               derivatives and virial: max|d| <= 1e-11 * max|ref|.  The
               per-pair arithmetic is the reference's (exp of DHENERGY is the
               device's, within an ulp); only the summation order differs.
"""
import numpy as np
import pytest

from plumed2_gb300.frames import jittered_lattice

pytestmark = pytest.mark.gpu


def _check(got, ref, s_scale, what=""):
    s, d, v = got
    s0, d0, v0 = ref
    assert abs(s - s0) <= 1e-12 * s_scale + 1e-300, (what, s, s0, s_scale)
    dscale = max(np.abs(d0).max(), 1e-300)
    assert np.abs(d - d0).max() <= 1e-11 * dscale, (what, np.abs(d - d0).max() / dscale)
    vscale = max(np.abs(v0).max(), 1e-300)
    assert np.abs(v - v0).max() <= 1e-11 * vscale, (what, np.abs(v - v0).max() / vscale)


def test_rt_dhenergy_golden(orc, golden):
    """regtest/basic/rt-dhenergy (and rt-dhenergy2's charge units) through the GPU."""
    import oracle
    from plumed2_gb300.action import DHEnergy
    g = golden("rt_dhenergy.json")
    q = np.array(g["charges"])
    pairs = orc.all_pairs(oracle.MODE_TWO, 3, 7)
    for ai, lab in enumerate(g["order"]):
        act = g["actions"][lab]
        line = "GROUPA=1-3 GROUPB=4-10 I=%r TEMP=%r EPSILON=%r" % (act["I"], act["TEMP"], act["EPSILON"])
        c = DHEnergy(line, charges=q)
        c2 = DHEnergy(line, charges=q / 0.1, units=(1.0, 1.0, 0.1))  # UNITS CHARGE=0.1
        k, cst = orc.dhenergy_constants(act["I"], act["TEMP"], act["EPSILON"])
        p = orc.pairing(oracle.CV_DHENERGY, charges=q, dh=(k, cst, act["EPSILON"]))
        pabs = orc.pairing(oracle.CV_DHENERGY, charges=np.abs(q), dh=(k, cst, act["EPSILON"]))
        for fi, (frame, box) in enumerate(zip(g["frames"], g["box"])):
            B = np.diag(box)
            s, d, v = c.calculate(np.array(frame), B)
            assert abs(s - g["colvar"][fi][ai]) <= 5.01e-6, (lab, fi)
            got = np.concatenate([d.reshape(-1), v.reshape(-1)])
            assert np.abs(got - np.array(g["deriv"][fi])[:, ai]).max() <= 5.01e-6, (lab, fi)
            assert abs(c2.calculate(np.array(frame), B)[0] - g["colvar_units_charge_0.1"][fi][ai]) <= 5.01e-6
            _check((s, d, v), orc.cv(p, frame, B, pairs), abs(orc.cv(pabs, frame, B, pairs)[0]), (lab, fi))


def test_rt_ghbfix_golden(orc, golden):
    """regtest/basic/rt-ghbfix through the GPU: 150 two-atom frames, PAIR."""
    import oracle
    from plumed2_gb300.action import GHBFIX
    g = golden("rt_ghbfix.json")
    c = GHBFIX(g["line"] + " TYPES=typesTable.dat PARAMS=scalingParameters.dat", types_text=g["types_file"],
               params_text=g["params_file"])
    p = orc.pairing(oracle.CV_GHBFIX, types=c.types[:2], eta=c.eta, ghbfix=(0.2, 0.3, 0.8))
    B = np.diag([100.0, 100.0, 100.0])
    for i in range(1, 151):
        z = float("%.6g" % (i * 0.002))
        pos = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, z]])
        s, d, v = c.calculate(pos, B)
        assert abs(s + g["c1_minus_ghbfix"] - g["colvar_c1"][i - 1]) <= 5.01e-5, i
        got = np.concatenate([d.reshape(-1), v.reshape(-1)])
        assert np.abs(got - np.array(g["deriv_ghbfix"][i - 1])).max() <= 5.01e-5, i
        ref = orc.cv(p, pos, B, np.array([[0, 1]], np.uint32))
        assert s == ref[0] and np.array_equal(d, ref[1]) and np.array_equal(v, ref[2]), i


def _groups(mode, n):
    if mode == "single":
        return "GROUPA=1-%d" % n, (0, n, 0)
    if mode == "two":
        return "GROUPA=1-%d GROUPB=%d-%d" % (n // 2, n // 2 + 1, n), (1, n // 2, n - n // 2)
    return "PAIR GROUPA=1-%d GROUPB=%d-%d" % (n // 2, n // 2 + 1, n), (2, n // 2, n // 2)


def _ref_pairs(orc, nl, m, n0, n1, pos, box, cut):
    if nl == "NLIST":
        return orc.nl_classic(m, n0, n1, pos, box, True, cut)
    if nl == "NLISTCELLS":
        return orc.nl_linkcells(m, n0, n1, pos, box, True, cut)
    return orc.all_pairs(m, n0, n1)


@pytest.mark.parametrize("mode", ["single", "two", "pair"])
@pytest.mark.parametrize("nl", ["", "NLIST", "NLISTCELLS"])
def test_dhenergy_parity(orc, mode, nl):
    import oracle
    from plumed2_gb300.action import DHEnergy
    if nl == "NLISTCELLS" and mode == "pair":
        pytest.skip("PAIR is not compatible with NLISTCELLS (CoordinationBase.cpp:72)")
    n = 1000
    pos = jittered_lattice(n, 0.30, 0.05, 11)
    box = np.diag([3.0] * 3)
    q = np.random.default_rng(5).uniform(-1.0, 1.0, n)
    grp, (m, n0, n1) = _groups(mode, n)
    line = grp + " I=0.15 TEMP=310 EPSILON=78.5" + (" %s NL_CUTOFF=0.9 NL_STRIDE=5" % nl if nl else "")
    c = DHEnergy(line, charges=q)
    got = c.calculate(pos, box, step=0)
    pairs = _ref_pairs(orc, nl, m, n0, n1, pos, box, 0.9)
    k, cst = orc.dhenergy_constants(0.15, 310.0, 78.5)
    ref = orc.cv(orc.pairing(oracle.CV_DHENERGY, charges=q, dh=(k, cst, 78.5)), pos, box, pairs)
    scale = orc.cv(orc.pairing(oracle.CV_DHENERGY, charges=np.abs(q), dh=(k, cst, 78.5)), pos, box, pairs)[0]
    _check(got, ref, scale, (mode, nl))


@pytest.mark.parametrize("mode", ["single", "two", "pair"])
@pytest.mark.parametrize("nl", ["", "NLIST", "NLISTCELLS"])
def test_ghbfix_parity(orc, mode, nl):
    """Three types, an asymmetric eta, and distances in every branch of the
    pairing (below D_0, the two polynomial pieces, beyond D_MAX)."""
    import oracle
    from plumed2_gb300.action import GHBFIX
    if nl == "NLISTCELLS" and mode == "pair":
        pytest.skip("PAIR is not compatible with NLISTCELLS (CoordinationBase.cpp:72)")
    n = 1000
    pos = jittered_lattice(n, 0.30, 0.06, 12)
    box = np.diag([3.0] * 3)
    rng = np.random.default_rng(6)
    names = ["O", "N", "H"]
    types_text = "#! FIELDS itype\n" + "".join(names[t] + "\n" for t in rng.integers(0, 3, n))
    eta = rng.uniform(-2.0, 2.0, (3, 3))
    params_text = "#! FIELDS itype jtype eta\n" + "".join(
        "%s %s %.17g\n" % (a, b, eta[i, j]) for i, a in enumerate(names) for j, b in enumerate(names))
    grp, (m, n0, n1) = _groups(mode, n)
    line = grp + " D_0=0.22 D_MAX=0.42 C=0.7 TYPES=t PARAMS=p" + (" %s NL_CUTOFF=0.6 NL_STRIDE=5" % nl if nl else "")
    c = GHBFIX(line, types_text=types_text, params_text=params_text)
    got = c.calculate(pos, box, step=0)
    pairs = _ref_pairs(orc, nl, m, n0, n1, pos, box, 0.6)
    slot_types = c.types[np.asarray(c.requested_atoms)]
    ref = orc.cv(orc.pairing(oracle.CV_GHBFIX, types=slot_types, eta=c.eta, ghbfix=(0.22, 0.42, 0.7)), pos, box,
                 pairs)
    scale = orc.cv(orc.pairing(oracle.CV_GHBFIX, types=slot_types, eta=np.abs(c.eta), ghbfix=(0.22, 0.42, 0.7)),
                   pos, box, pairs)[0]
    _check(got, ref, abs(scale), (mode, nl))


def test_sibling_backward_and_saved_forward():
    """dV/dx from the backward kernel (recomputing) and from a saved forward
    equal g * ds/dx of the forward, batched over frames."""
    import torch
    from plumed2_gb300 import _lib
    from plumed2_gb300.action import DHEnergy
    n, F = 800, 3
    frames = np.stack([jittered_lattice(n, 0.30, 0.05, 20 + f) for f in range(F)])
    boxes = np.stack([np.diag([2.8] * 3)] * F)
    q = np.random.default_rng(7).uniform(-1.0, 1.0, n)
    c = DHEnergy("GROUPA=1-%d I=0.1 NLIST NL_CUTOFF=1.0 NL_STRIDE=10" % n, charges=q)
    dev = torch.device("cuda:0")
    pos = torch.from_numpy(frames).to(dev)
    s = torch.zeros(F, dtype=torch.float64, device=dev)
    der = torch.zeros(F, n, 3, dtype=torch.float64, device=dev)
    vir = torch.zeros(F, 9, dtype=torch.float64, device=dev)
    c.forward_device(pos.data_ptr(), boxes, F, s.data_ptr(), der.data_ptr(), vir.data_ptr(), step=0)
    g = torch.tensor([0.5, -1.25, 2.0], dtype=torch.float64, device=dev)
    gp = torch.zeros(F, n, 3, dtype=torch.float64, device=dev)
    c.backward_device(pos.data_ptr(), boxes, F, g.data_ptr(), gp.data_ptr())
    want = (g[:, None, None] * der).cpu().numpy()
    assert np.abs(gp.cpu().numpy() - want).max() <= 1e-12 * np.abs(want).max()
    c.forward_device(pos.data_ptr(), boxes, F, s.data_ptr(), 0, vir.data_ptr(), step=1, flags=_lib.FLAG_SAVE)
    gp2 = torch.zeros_like(gp)
    c.backward_device(pos.data_ptr(), boxes, F, g.data_ptr(), gp2.data_ptr())
    assert np.abs(gp2.cpu().numpy() - want).max() <= 1e-12 * np.abs(want).max()


def test_sibling_refusals():
    from plumed2_gb300 import _lib
    from plumed2_gb300._lib import CoordError
    from plumed2_gb300.action import Coordination, DHEnergy, GHBFIX
    pos = jittered_lattice(64, 0.3, 0.03, 1)
    box = np.diag([1.2] * 3)
    # no charges given
    c = DHEnergy("GROUPA=1-64")
    with pytest.raises(CoordError) as e:
        c.calculate(pos, box)
    assert e.value.status == _lib.COORD_ERR_STATE
    # charges that do not cover the group
    c.set_charges(np.ones(10))
    with pytest.raises(CoordError, match="atom number 11"):
        c.calculate(pos, box)
    c.set_charges(np.ones(64))
    c.calculate(pos, box)
    # R_0/D_0 derivatives belong to COORDINATION
    s1, d1, v1 = np.zeros(1), np.zeros((64, 3)), np.zeros(9)
    with pytest.raises(CoordError) as e:
        c.forward_host(pos.ctypes.data, box.ctypes.data, 0, _lib.FLAG_DR0, s1.ctypes.data, d1.ctypes.data,
                       v1.ctypes.data)
    assert e.value.status == _lib.COORD_ERR_UNSUPPORTED
    # the types table must cover the group (GHBFIX.cpp:181-186)
    g = GHBFIX("GROUPA=1-64 D_0=0.2 D_MAX=0.3 C=0.8", types_text="#! FIELDS itype\nA\nB\n",
               params_text="#! FIELDS itype jtype eta\nA B 1.0\n")
    with pytest.raises(CoordError, match="your types table only covers 2 atoms, but you are trying to access atom "
                                         "number 3"):
        g.calculate(pos, box)
    with pytest.raises(ValueError, match="D_MAX is compulsory"):
        GHBFIX("GROUPA=1-64 D_0=0.2 C=0.8", types_text="", params_text="")
    with pytest.raises(ValueError, match="cannot read keyword SWITCH"):
        DHEnergy("GROUPA=1-64 SWITCH={RATIONAL R_0=1}")
    # the mixed path evaluates COORDINATION's switching function only
    cm = Coordination("GROUPA=1-64 R_0=0.3", precision="mixed")
    L = cm._L
    assert L.coord_set_dhenergy(cm._ctx, 0.1, 300.0, 80.0, 1.0, 1.0, 1.0) == _lib.COORD_ERR_UNSUPPORTED
