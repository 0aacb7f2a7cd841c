"""CONTACTMAP on the GPU against the reference's regtest goldens (rt28, rt72)
and the FP64 oracle.

Tolerances: the goldens' print formats (%f, %8.6f, %12.8f); against the
oracle, max|d| <= 1e-12 max|ref| for values, derivatives and virials (the
per-contact arithmetic is the reference's; the device's exp and the order of
the SUM/CMDIST reduction differ).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _line(m):
    parts = []
    for i, c in enumerate(m["contacts"], 1):
        parts.append("ATOMS%d=%d,%d SWITCH%d={%s} REFERENCE%d=%r WEIGHT%d=%r" % (
            i, c["atoms"][0], c["atoms"][1], i, c["switch"], i, c["reference"], i, c["weight"]))
    if m["sum"]:
        parts.append("SUM")
    if m["cmdist"]:
        parts.append("CMDIST")
    return " ".join(parts)


def _close(a, b, tol, what=""):
    a, b = np.asarray(a, float), np.asarray(b, float)
    assert np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300), (what, np.abs(a - b).max())


def test_rt28_golden(orc, golden):
    from plumed2_gb300.action import ContactMap
    r = golden("rt_contactmap.json")["rt28"]
    idx = {a: k for k, a in enumerate(r["atoms"])}
    ma, mc = r["maps"]
    a, c = ContactMap(_line(ma)), ContactMap(_line(mc))
    for fi, (fr, bx) in enumerate(zip(r["frames"], r["box"])):
        B = np.diag(bx)
        pa = np.array([fr[idx[x + 1]] for x in a.requested_atoms])  # 0-based indices, 1-based serials
        pc = np.array([fr[idx[x + 1]] for x in c.requested_atoms])
        va, da, wa = a.calculate(pa, B)
        vc, dc, wc = c.calculate(pc, B)
        assert abs(va - r["colvar"][fi][0]) <= 5.01e-7
        assert abs(vc[0] - r["colvar"][fi][1]) <= 5.01e-7 and abs(vc[4] - r["colvar"][fi][2]) <= 5.01e-7
        got = np.concatenate([da.reshape(-1), wa.reshape(-1)])
        assert np.abs(got - np.array(r["deriv_a"][fi])).max() <= 5.01e-7, fi
        # and against the oracle, tightly
        sw = [x["switch"] for x in ma["contacts"]]
        ov, od, ow = orc.contactmap(sw, pa, B, [x["reference"] for x in ma["contacts"]],
                                    [x["weight"] for x in ma["contacts"]], 2)
        _close(va, ov[0], 1e-12)
        _close(da, od, 1e-12)
        _close(wa, ow, 1e-12)
        ov, od, ow = orc.contactmap([x["switch"] for x in mc["contacts"]], pc, B, None, None, 0)
        _close(vc, ov, 1e-12)
        _close(dc, od, 1e-12)
        _close(wc, ow, 1e-12)


def test_rt72_golden_triclinic(orc, golden):
    from plumed2_gb300.action import ContactMap
    r = golden("rt_contactmap.json")["rt72"]
    cm = ContactMap(_line(r["map"]))
    P = np.array(r["pos"])
    pos = P[np.array(cm.requested_atoms)]
    B = np.array(r["box"]).reshape(3, 3)
    v, d, w = cm.calculate(pos, B)
    assert abs(v - r["value"]) <= 5.01e-7
    got = np.concatenate([d.reshape(-1), w.reshape(-1)])
    assert np.abs(got - np.array(r["deriv"])).max() <= 5.01e-9
    cs = r["map"]["contacts"]
    ov, od, ow = orc.contactmap([x["switch"] for x in cs], pos, B, [x["reference"] for x in cs],
                                [x["weight"] for x in cs], 1)
    _close(v, ov[0], 1e-12)
    _close(d, od, 1e-12)
    _close(w, ow, 1e-12)


@pytest.mark.parametrize("mode", ["", "SUM", "CMDIST"])
def test_contactmap_batched_parity(orc, mode):
    """2,000 random contacts among 3,000 atoms, a different switch per contact
    (RATIONAL, EXP, GAUSSIAN, SMAP, TANH), three frames in one launch."""
    import torch
    from plumed2_gb300 import _lib
    from plumed2_gb300.action import ContactMap
    rng = np.random.default_rng(8)
    n, natoms, F = 2000, 3000, 3
    kinds = ["RATIONAL R_0=%.3f NN=%d MM=%d D_MAX=%.3f", "EXP R_0=%.3f D_0=0.05", "GAUSSIAN R_0=%.3f",
             "SMAP R_0=%.3f A=3 B=5", "TANH R_0=%.3f"]
    parts, sws, refs, ws = [], [], [], []
    for i in range(1, n + 1):
        a, b = rng.choice(natoms, 2, replace=False) + 1
        k = i % len(kinds)
        r0 = rng.uniform(0.2, 0.6)
        sw = kinds[k] % ((r0, 6 + 2 * (i % 3), 12 + 2 * (i % 5), 2.5 * r0) if k == 0 else (r0,))
        ref, w = rng.uniform(0, 1), rng.uniform(0.5, 2)
        parts.append("ATOMS%d=%d,%d SWITCH%d={%s} REFERENCE%d=%.17g WEIGHT%d=%.17g" % (i, a, b, i, sw, i, ref, i, w))
        sws.append(sw)
        refs.append(ref)
        ws.append(w)
    cm = ContactMap(" ".join(parts) + (" " + mode if mode else ""))
    L = 4.0
    frames = rng.uniform(0, L, (F, natoms, 3))
    boxes = np.stack([np.diag([L, L * 1.1, L * 0.9])] * F)
    req = np.array(cm.requested_atoms)
    pos = np.ascontiguousarray(frames[:, req, :])
    dev = torch.device("cuda:0")
    tp = torch.as_tensor(pos, device=dev)
    nv = n if cm.mode == _lib.CMAP_COMPONENTS else 1
    value = torch.empty(F, nv, dtype=torch.float64, device=dev)
    deriv = torch.empty(F, 2 * n, 3, dtype=torch.float64, device=dev)
    vir = torch.empty(F, nv, 9, dtype=torch.float64, device=dev)
    cm.forward_device(tp.data_ptr(), boxes, F, value.data_ptr(), deriv.data_ptr(), vir.data_ptr())
    value, deriv, vir = value.cpu().numpy(), deriv.cpu().numpy(), vir.cpu().numpy()
    for f in range(F):
        ov, od, ow = orc.contactmap(sws, pos[f], boxes[f], refs, ws, cm.mode)
        _close(value[f], ov, 1e-12, (mode, f))
        _close(deriv[f], od, 1e-12, (mode, f))
        _close(vir[f].reshape(ow.shape), ow, 1e-12, (mode, f))


def test_contactmap_refusals():
    from plumed2_gb300._lib import CoordError
    from plumed2_gb300.action import ContactMap
    with pytest.raises(CoordError, match="SWITCH"):
        ContactMap("ATOMS1=1,2 SWITCH={CUSTOM FUNC=1/(1+x^6) R_0=1}")
    with pytest.raises(ValueError, match="REFERENCE"):
        ContactMap("ATOMS1=1,2 SWITCH={RATIONAL R_0=1} CMDIST")
