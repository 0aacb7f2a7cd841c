"""GPU results (through the C ABI) against the FP64 oracle on the same inputs.

Tolerances, stated here once:
  FP64 path   s: |ds|/|s| <= 1e-12;  derivatives and virial: max|d| / max|ref| <= 1e-11
              (the per-pair arithmetic is the reference's; only the summation
              order differs -- atomics and tree reductions)
  mixed path  s: |ds|/|s| <= 1e-6;   derivatives: max_i|dF_i| / max_i|F_i| <= 1e-5;
              virial: max|dW| / max|W| <= 1e-5
  neighbour lists: the pair set is bit-exact (sorted comparison).
"""
import json
import os

import numpy as np
import pytest

from plumed2_gb300.frames import jittered_lattice

pytestmark = pytest.mark.gpu

TOL = {"fp64": (1e-12, 1e-11), "mixed": (1e-6, 1e-5)}


def _check(prec, got, ref, what="", dfloor=1e-300):
    """dfloor: least derivative scale (frames on a perfect lattice, whose
    derivatives cancel atom by atom, take the size of their virial)."""
    s, d, v = got
    s0, d0, v0 = ref
    ts, td = TOL[prec]
    assert abs(s - s0) <= ts * max(abs(s0), 1e-300) + 1e-300, (what, s, s0)
    dscale = max(np.abs(d0).max(), dfloor)
    assert np.abs(d - d0).max() <= td * dscale, (what, np.abs(d - d0).max() / dscale)
    vscale = max(np.abs(v0).max(), 1e-300)
    assert np.abs(v - v0).max() <= td * vscale, (what, np.abs(v - v0).max() / vscale)


def _sorted(p):
    p = np.asarray(p).reshape(-1, 2)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def _abs_index(c):
    return np.asarray(c.requested_atoms, dtype=np.int64)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("pbc", [True, False])
def test_allpairs_single(orc, prec, pbc):
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.30 D_0=0.0 NN=6 MM=12 D_MAX=1.0"
    pos = jittered_lattice(1000, 0.30, 0.03, 1)
    box = np.diag([3.0] * 3)
    c = Coordination("GROUPA=1-1000 SWITCH={%s}%s" % (spec, "" if pbc else " NOPBC"), precision=prec)
    got = c.calculate(pos, box)
    ref = orc.coordination(spec, pos, box, orc.all_pairs(0, 1000), do_pbc=pbc)
    _check(prec, got, ref)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_allpairs_twolist_and_self_pairs(orc, prec):
    """GROUPA and GROUPB overlap: pairs of the same atom are skipped."""
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.35 NN=6 MM=12 D_MAX=1.2"
    sysp = jittered_lattice(900, 0.31, 0.03, 2)
    box = np.diag([0.31 * 10] * 3)
    c = Coordination("GROUPA=1-600 GROUPB=301-900 SWITCH={%s}" % spec, precision=prec)
    pos = sysp[c.requested_atoms]
    got = c.calculate(pos, box)
    ref = orc.coordination(spec, pos, box, orc.all_pairs(1, 600, 600), abs_index=_abs_index(c))
    _check(prec, got, ref)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_r0_syntax_default_switch(orc, prec):
    from plumed2_gb300.action import Coordination
    pos = jittered_lattice(343, 0.3, 0.03, 3)
    box = np.diag([2.1] * 3)
    c = Coordination("GROUPA=1-343 R_0=0.3", precision=prec)
    got = c.calculate(pos, box)
    ref = orc.coordination("R0SYNTAX 6 0 0.3 0.0", pos, box, orc.all_pairs(0, 343))
    _check(prec, got, ref)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("mode", ["single", "two"])
@pytest.mark.parametrize("pbc", [True, False])
def test_nlist_semantics_over_steps(orc, prec, mode, pbc):
    """NLIST: pair set bit-exact at each rebuild; between rebuilds the list of
    the last rebuild is evaluated at the new positions (NeighborList::prepare)."""
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.35 NN=6 MM=12 D_MAX=1.0"
    n = 4096
    L = 16 * 0.31
    box = np.diag([L] * 3)
    if mode == "single":
        line, m, n0, n1 = "GROUPA=1-4096", 0, n, 0
    else:
        line, m, n0, n1 = "GROUPA=1-2048 GROUPB=2049-4096", 1, 2048, 2048
    c = Coordination("%s SWITCH={%s} NLIST NL_CUTOFF=0.9 NL_STRIDE=3%s" % (line, spec, "" if pbc else " NOPBC"),
                     precision=prec)
    rng = np.random.default_rng(5)
    pos = jittered_lattice(n, 0.31, 0.03, 4)
    nl_ref = None
    for step in range(7):
        if step % 3 == 0:
            nl_ref = orc.nl_classic_cells(m, n0, n1, pos, box, pbc, 0.9)
        got = c.calculate(pos, box, step)
        if step % 3 == 0:
            assert np.array_equal(_sorted(c.pairs()), nl_ref), step
            assert c.nl_size() == len(nl_ref)
        ref = orc.coordination(spec, pos, box, nl_ref, do_pbc=pbc)
        _check(prec, got, ref, "step %d" % step)
        pos = pos + rng.normal(0, 0.01, pos.shape)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("mode", ["single", "two"])
@pytest.mark.parametrize("pbc", [True, False])
def test_nlist_pairs_crossing_dmax_between_rebuilds(orc, prec, mode, pbc):
    """D_MAX below NL_CUTOFF: steps of 0.04 nm per coordinate between rebuilds
    carry thousands of listed pairs across D_MAX both ways (1,273 into it
    after one step, 5,831 after three).  s, the derivatives and the virial
    follow the oracle on the last rebuild's list at each step, and the pair
    set is the oracle's at each rebuild."""
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.3 NN=6 MM=12 D_MAX=0.6"
    n = 4096
    L = 16 * 0.31
    box = np.diag([L] * 3)
    if mode == "single":
        line, m, n0, n1 = "GROUPA=1-4096", 0, n, 0
    else:
        line, m, n0, n1 = "GROUPA=1-2048 GROUPB=2049-4096", 1, 2048, 2048
    c = Coordination("%s SWITCH={%s} NLIST NL_CUTOFF=0.9 NL_STRIDE=4%s" % (line, spec, "" if pbc else " NOPBC"),
                     precision=prec)
    rng = np.random.default_rng(11)
    pos = jittered_lattice(n, 0.31, 0.03, 6)
    nl_ref = None
    for step in range(9):
        if step % 4 == 0:
            nl_ref = orc.nl_classic_cells(m, n0, n1, pos, box, pbc, 0.9)
        got = c.calculate(pos, box, step)
        if step % 4 == 0:
            assert np.array_equal(_sorted(c.pairs()), nl_ref), step
            assert c.nl_size() == len(nl_ref)
        ref = orc.coordination(spec, pos, box, nl_ref, do_pbc=pbc)
        _check(prec, got, ref, "step %d" % step)
        pos = pos + rng.normal(0, 0.04, pos.shape)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["NLIST", "NLISTCELLS"])
@pytest.mark.parametrize("mode", ["single", "two"])
def test_near_and_far_rows_over_a_trajectory(orc, prec, kind, mode):
    """Lists of orthorhombic periodic frames are split at each rebuild into a
    near part (within D_MAX + skin) and a far part; while every atom has
    moved less than half the skin since the rebuild only the near parts are
    read.  A trajectory of small steps (0.002 nm per coordinate) over three
    NL_STRIDE=10 intervals, with one kick of 0.08 nm at step 14 that moves
    atoms past half the skin (the far parts are read again until the next
    rebuild), and a box that changes at step 23 (no near parts until the
    next rebuild).  Every step follows the oracle on the last rebuild's
    list."""
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.3 NN=6 MM=12 D_MAX=0.6"
    n, a0 = 4096, 0.31
    L = 16 * a0
    if mode == "single":
        line, m, n0, n1 = "GROUPA=1-4096", 0, n, 0
    else:
        line, m, n0, n1 = "GROUPA=1-2048 GROUPB=2049-4096", 1, 2048, 2048
    c = Coordination("%s SWITCH={%s} %s NL_CUTOFF=0.8 NL_STRIDE=10" % (line, spec, kind), precision=prec)
    rng = np.random.default_rng(21)
    pos = jittered_lattice(n, a0, 0.03, 9)
    nl_ref = None
    for step in range(30):
        box = np.diag([L] * 3) if step < 23 else np.diag([L * 1.001] * 3)
        if step % 10 == 0:
            if kind == "NLIST":
                nl_ref = orc.nl_classic_cells(m, n0, n1, pos, box, True, 0.8)
            else:
                nl_ref = orc.nl_linkcells(m, n0, n1, pos, box, True, 0.8)
        got = c.calculate(pos, box, step)
        if step % 10 == 0:
            assert np.array_equal(_sorted(c.pairs()), _sorted(nl_ref)), step
        ref = orc.coordination(spec, pos, box, nl_ref)
        _check(prec, got, ref, "step %d" % step)
        pos = pos + rng.normal(0, 0.08 if step == 14 else 0.002, pos.shape)


@pytest.mark.parametrize("mode", ["single", "two"])
@pytest.mark.parametrize("pbc", [True, False])
def test_nlistcells_pair_set(orc, mode, pbc):
    """NLISTCELLS: every pair of neighbouring link cells (LinkCells geometry)."""
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.35 NN=6 MM=12 D_MAX=0.8"
    pos = jittered_lattice(1728, 0.31, 0.03, 6)
    box = np.diag([12 * 0.31] * 3)
    if mode == "single":
        line, m, n0, n1 = "GROUPA=1-1728", 0, 1728, 0
    else:
        line, m, n0, n1 = "GROUPA=1-864 GROUPB=865-1728", 1, 864, 864
    c = Coordination("%s SWITCH={%s} NLISTCELLS NL_CUTOFF=0.8 NL_STRIDE=2%s" % (line, spec, "" if pbc else " NOPBC"))
    got = c.calculate(pos, box, 0)
    ref_pairs = orc.nl_linkcells(m, n0, n1, pos, box, pbc, 0.8)
    assert np.array_equal(_sorted(c.pairs()), _sorted(ref_pairs))
    ref = orc.coordination(spec, pos, box, ref_pairs, do_pbc=pbc)
    _check("fp64", got, ref)


@pytest.mark.parametrize("pbc", [True, False])
def test_nlistcells_refuses_box_without_volume(orc, pbc):
    """LinkCells::setupCells(pbc) (LinkCells.cpp:75-83): a cell list on a box
    whose volume is not above DBL_EPSILON (here a left-handed one) is refused
    at the rebuild with the reference's message, with or without NOPBC (the
    list gets the box either way).  The context then builds on a proper box."""
    from plumed2_gb300 import CoordError, _lib
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.35 NN=6 MM=12 D_MAX=0.8"
    pos = jittered_lattice(1728, 0.31, 0.03, 6)
    L = 12 * 0.31
    c = Coordination("GROUPA=1-1728 SWITCH={%s} NLISTCELLS NL_CUTOFF=0.8 NL_STRIDE=2%s" % (spec, "" if pbc else " NOPBC"))
    left = np.array([[0.0, L, 0.0], [L, 0.0, 0.0], [0.0, 0.0, L]])
    with pytest.raises(CoordError, match="Cell lists cannot be built when passing a box with null volume") as e:
        c.calculate(pos, left, 0)
    assert e.value.status == _lib.COORD_ERR_BOX
    box = np.diag([L] * 3)
    got = c.calculate(pos, box, 0)
    ref_pairs = orc.nl_linkcells(0, 1728, 0, pos, box, pbc, 0.8)
    assert np.array_equal(_sorted(c.pairs()), _sorted(ref_pairs))
    _check("fp64", got, orc.coordination(spec, pos, box, ref_pairs, do_pbc=pbc))


@pytest.mark.parametrize("variant", ["rt42-cells", "rt42-cells-cos", "rt42-cells-gauss"])
def test_rt42_cells_golden(orc, golden, variant):
    """regtest/basic/rt42-cells{,-cos,-gauss} through the C ABI: the NLIST and
    NLISTCELLS actions of each input (GROUPA=GROUPB=1-108, triclinic box,
    NL_STRIDE=4) over the 27 frames.  d - c against check_diff.reference
    (%8.4f), the forces and virial of SLOPE=0.001 on d - c against
    ff.reference (%10.5f, all zero), and each action against the oracle on
    the lists of its own last rebuild (FP64 tolerances above; every frame is
    a perfect lattice, so the derivatives cancel atom by atom and the virial's
    size is their scale)."""
    from plumed2_gb300.action import Coordination
    import re
    g = golden("rt42_cells.json")
    v = g["variants"][variant]
    spec = re.search(r"SWITCH=\{([^}]*)\}", v["c"]).group(1).strip()
    c, d = Coordination(v["c"]), Coordination(v["d"])
    n = 108
    absi = _abs_index(c)
    assert np.array_equal(absi, _abs_index(d))
    for step, (fr, bx) in enumerate(zip(g["frames"], g["box"])):
        pos = np.array(fr)[absi]
        box = np.array(bx).reshape(3, 3)
        if step % 4 == 0:
            pc = orc.nl_classic(1, n, n, pos, box, True, 2.0)
            pd = orc.nl_linkcells(1, n, n, pos, box, True, 2.0)
        got_c = c.calculate(pos, box, step)
        got_d = d.calculate(pos, box, step)
        for got, pairs, lab in ((got_c, pc, "c"), (got_d, pd, "d")):
            ref = orc.coordination(spec, pos, box, pairs, abs_index=absi)
            _check("fp64", got, ref, "%s step %d" % (lab, step), dfloor=np.abs(ref[2]).max())
        assert abs((got_d[0] - got_c[0]) - v["check_diff"][step]) <= 5.01e-5, step
        fd = np.zeros((n, 3))
        np.add.at(fd, absi, 0.001 * (got_d[1] - got_c[1]))
        assert np.abs(fd).max() <= 5.01e-6 and np.abs(0.001 * (got_d[2] - got_c[2])).max() <= 5.01e-6, step


def _oracle_spec(line):
    """The oracle's switch spec of a COORDINATION line: the SWITCH={...}
    definition, or the R_0/NN/MM/D_0 keywords (defaults NN=6, MM=0 -> 2NN,
    D_0=0)."""
    import re
    m = re.search(r"SWITCH=\{([^}]*)\}", line)
    if m:
        return m.group(1).strip()
    kw = dict(re.findall(r"\b(R_0|NN|MM|D_0)=(\S+)", line))
    return "R0SYNTAX %s %s %s %s" % (kw.get("NN", "6"), kw.get("MM", "0"), kw["R_0"], kw.get("D_0", "0.0"))


with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cudacoord_plugin.json")) as _f:
    _CUDACOORD_CASES = sorted(json.load(_f)["cases"])


@pytest.mark.parametrize("case", _CUDACOORD_CASES)
def test_cudacoord_plugin_regtests(orc, golden, case):
    """plugins/cudaCoord/regtest: each input of the reference's CUDA plugin
    tests, whose COORDINATION twin printed gpu - cpu = 0 at %8.4f and
    derivative deltas of 0 at %8.5f, run here through the C ABI over its ten
    frames and compared with the oracle (the reference's CPU arithmetic):
    within those print tolerances, and within this file's FP64 or mixed
    tolerances (the rt-float-* inputs on the mixed path)."""
    from plumed2_gb300.action import Coordination
    g = golden("cudacoord_plugin.json")
    cs = g["cases"][case]
    tr = g["trajectories"][cs["traj"]]
    prec = "mixed" if cs["float"] else "fp64"
    c = Coordination(cs["line"], precision=prec)
    absi = _abs_index(c)
    na, nb = len(c.group_a), len(c.group_b)
    mode = 2 if " PAIR" in " " + cs["line"] else (1 if nb else 0)
    pairs = orc.all_pairs(mode, na, nb) if mode else orc.all_pairs(0, na)
    spec = _oracle_spec(cs["line"])
    assert cs["deriv_delta_max"] == 0.0 and max(map(abs, cs["diff"])) == 0.0
    for step, (fr, bx) in enumerate(zip(tr["frames"], tr["box"])):
        pos = np.array(fr)[absi]
        box = np.array(bx).reshape(3, 3)
        got = c.calculate(pos, box, step)
        ref = orc.coordination(spec, pos, box, pairs, abs_index=absi, do_pbc=" NOPBC" not in " " + cs["line"])
        assert abs(got[0] - ref[0]) <= 5.01e-5, (case, step)
        assert np.abs(got[1] - ref[1]).max() <= 5.01e-6, (case, step)
        _check(prec, got, ref, "%s step %d" % (case, step), dfloor=np.abs(ref[2]).max())


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("nl", [False, True])
def test_pair_mode(orc, prec, nl):
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.35 NN=6 MM=12 D_MAX=1.5"
    pos = jittered_lattice(1000, 0.30, 0.05, 7)
    box = np.diag([3.0] * 3)
    extra = " NLIST NL_CUTOFF=1.0 NL_STRIDE=1" if nl else ""
    c = Coordination("GROUPA=1-500 GROUPB=501-1000 PAIR SWITCH={%s}%s" % (spec, extra), precision=prec)
    got = c.calculate(pos, box)
    pairs = orc.nl_classic(2, 500, 500, pos, box, True, 1.0) if nl else orc.all_pairs(2, 500, 500)
    if nl:
        assert np.array_equal(_sorted(c.pairs()), _sorted(pairs))
    ref = orc.coordination(spec, pos, box, pairs)
    _check(prec, got, ref)


SWITCHES = ["RATIONAL R_0=0.3 NN=5 MM=11 D_MAX=0.9", "RATIONAL R_0=0.3 NN=5 D_MAX=0.9",
            "RATIONAL R_0=0.3 NN=6 MM=10 D_MAX=0.9", "RATIONAL R_0=0.3 NN=8 MM=16 D_MAX=0.9",
            "RATIONAL R_0=0.3 NN=6 MM=12", "EXP R_0=0.2 D_0=0.1 D_MAX=0.9", "GAUSSIAN R_0=1.0 D_0=0.0 D_MAX=0.9",
            "GAUSSIAN R_0=0.3 D_0=0.1 D_MAX=0.9", "TANH R_0=0.3 D_MAX=0.9", "SMAP R_0=0.3 A=3 B=2 D_MAX=0.9",
            "CUBIC D_MAX=0.9 D_0=0.1", "COSINUS R_0=0.9", "Q R_0=0.3 D_0=0.1 BETA=5.0 LAMBDA=1.0 REF=0.4 D_MAX=0.9",
            "CUSTOM FUNC=1/(1+x^6) R_0=0.3 D_MAX=0.9", "CUSTOM FUNC=1/(1+x2^3) R_0=0.3 D_MAX=0.9",
            "CUSTOM FUNC=exp(-x^2)*cos(x) R_0=0.3 D_0=0.05 D_MAX=0.9",
            "CUSTOM FUNC=step(1-x)*(1-x)^2+0.1*tanh(1-x) R_0=0.4 D_MAX=0.9"]


@pytest.mark.parametrize("spec", SWITCHES)
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_switch_types(orc, spec, prec):
    from plumed2_gb300.action import Coordination
    pos = jittered_lattice(512, 0.3, 0.04, 8)
    box = np.diag([2.4] * 3)
    c = Coordination("GROUPA=1-512 SWITCH={%s}" % spec, precision=prec)
    got = c.calculate(pos, box)
    ref = orc.coordination(spec, pos, box, orc.all_pairs(0, 512))
    prec_t = prec
    if prec == "fp64" and not spec.startswith("RATIONAL"):
        # CUDA's exp/tanh/cos/pow may differ from the host libm in the last ulp
        TOL["fp64_libm"] = (1e-11, 1e-10)
        prec_t = "fp64_libm"
    _check(prec_t, got, ref)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_custom_switch_nlist_steps(orc, prec):
    """CUSTOM switches through the neighbour-list path, lists rebuilt every
    second step while the atoms move, against the oracle on the same list."""
    from plumed2_gb300.action import Coordination
    rng = np.random.default_rng(11)
    pos = jittered_lattice(1000, 0.3, 0.03, 10)
    box = np.diag([3.0] * 3)
    spec = "CUSTOM FUNC=exp(-x^2)*cos(x) R_0=0.3 D_0=0.05 D_MAX=0.8"
    c = Coordination("GROUPA=1-1000 SWITCH={%s} NLIST NL_CUTOFF=1.0 NL_STRIDE=2" % spec, precision=prec)
    tol = "fp64_libm" if prec == "fp64" else prec
    TOL["fp64_libm"] = (1e-11, 1e-10)
    for step in range(4):
        if step % 2 == 0:
            pairs = orc.nl_classic(0, 1000, 0, pos, box, True, 1.0)
        got = c.calculate(pos, box, step)
        if step % 2 == 0:
            assert np.array_equal(_sorted(c.pairs()), _sorted(pairs)), step
        _check(tol, got, orc.coordination(spec, pos, box, pairs), step)
        pos = pos + rng.normal(0.0, 0.01, pos.shape)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_triclinic_box_rt42_golden(orc, golden, prec):
    """regtest/basic/rt42 through the GPU: a triclinic box that the reference
    reduces, GROUPA and GROUPB the same 108 atoms; values at %8.4f,
    forces/virial at %10.5f (the regtest's own precision; for the mixed path
    that plus its relative bounds: the values are about 1.2e4 and the
    virial about 620 on the diagonal), with d,
    dfast, f and h the regtest's own CUSTOM (lepton) switching functions."""
    from plumed2_gb300.action import Coordination
    g = golden("rt42.json")
    cs = {k: Coordination("GROUPA=1-108 GROUPB=1-108 " + v, precision=prec) for k, v in [
        ("c", "R_0=1"), ("d", "SWITCH={CUSTOM FUNC=1/(1+x^6) R_0=1}"),
        ("dfast", "SWITCH={CUSTOM FUNC=1/(1+x2^3) R_0=1}"), ("e", "R_0=1 NN=7 D_0=0.1"),
        ("f", "SWITCH={CUSTOM FUNC=1/(1+x^7) R_0=1 D_0=0.1}"), ("g", "SWITCH={EXP R_0=1}"),
        ("h", "SWITCH={CUSTOM FUNC=exp(-x) R_0=1}")]}
    c1 = Coordination("GROUPA=1-108 R_0=1", precision=prec)
    for fi in range(len(g["frames"])):
        pos = np.array(g["frames"][fi])
        box = np.array(g["box"][fi]).reshape(3, 3)
        n = len(pos)
        o = {}
        for k, c in cs.items():
            s, d, v = c.calculate(np.concatenate([pos, pos]), box)
            o[k] = (s, d[:n] + d[n:], v)
        for k in "ceg":
            # mixed: the printed precision plus the path's relative bound
            tol = 5.01e-5 + (TOL[prec][0] * abs(g[k][fi]) if prec == "mixed" else 0.0)
            assert abs(o[k][0] - g[k][fi]) <= tol, (fi, k)
        for i in (1, 2):
            X = -(o["c"][i] + o["d"][i]) - 0.001 * (o["c"][i] - 0.5 * o["d"][i] - 0.5 * o["dfast"][i]
                                                    + o["e"][i] - o["f"][i] + o["g"][i] - o["h"][i])
            ref = np.array(g["ff_forces" if i == 1 else "ff_virial"][fi]).reshape(X.shape)
            # mixed: the printed precision plus the path's relative bound (the
            # virial's diagonal is about 620)
            tol = 5.01e-6 + (TOL[prec][1] * np.abs(ref).max() if prec == "mixed" else 0.0)
            assert np.abs(X - ref).max() <= tol, (fi, i, np.abs(X - ref).max())
        tol = 5.01e-5 + (TOL[prec][0] * abs(g["c_single"][fi]) if prec == "mixed" else 0.0)
        assert abs(c1.calculate(pos, box)[0] - g["c_single"][fi]) <= tol


TRIC_BOX = np.array([[3.0, 0.0, 0.0], [0.9, 2.8, 0.0], [-0.6, 0.7, 2.9]])


def _tric_frame(m, box, sigma, seed):
    """m^3 atoms on a jittered lattice in scaled coordinates, through the box rows."""
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*(np.arange(m),) * 3, indexing="ij"), -1).reshape(-1, 3)
    return ((g + 0.5) / m + rng.normal(0.0, sigma, g.shape)) @ box


@pytest.mark.parametrize("kind", ["none", "NLIST", "NLISTCELLS", "PAIR", "PAIR+NLIST"])
@pytest.mark.parametrize("groups", ["single", "two"])
def test_mixed_triclinic_box(orc, kind, groups):
    """The mixed path on a triclinic box: FP32 pair geometry through the
    reduced cell (and its octant shifts), the D_MAX band decided in FP64;
    pair sets bit-exact, values within the mixed tolerance of the oracle."""
    from plumed2_gb300.action import Coordination
    if groups == "single" and kind.startswith("PAIR"):
        pytest.skip("PAIR needs two groups")
    spec = "RATIONAL R_0=0.3 NN=6 MM=12 D_MAX=0.9"
    pos = _tric_frame(10, TRIC_BOX, 0.01, 3)
    n = len(pos)
    if groups == "single":
        line, m, n0, n1 = "GROUPA=1-1000", 0, n, 0
    else:
        line, m, n0, n1 = "GROUPA=1-500 GROUPB=501-1000", 1, 500, 500
    if kind.startswith("PAIR"):
        line += " PAIR"
        m = 2
        pos = np.concatenate([pos[:500], pos[100:600]])  # pair i: lattice neighbours along the first row
    nl = {"NLIST": " NLIST NL_CUTOFF=1.1 NL_STRIDE=2", "NLISTCELLS": " NLISTCELLS NL_CUTOFF=1.1 NL_STRIDE=2",
          "PAIR+NLIST": " NLIST NL_CUTOFF=1.1 NL_STRIDE=1"}.get(kind, "")
    c = Coordination("%s SWITCH={%s}%s" % (line, spec, nl), precision="mixed")
    rng = np.random.default_rng(9)
    for step in range(3):
        got = c.calculate(pos, TRIC_BOX, step)
        if kind == "NLISTCELLS":
            if step % 2 == 0:
                pairs = orc.nl_linkcells(m, n0, n1, pos, TRIC_BOX, True, 1.1)
        elif nl:
            if step % 2 == 0 or kind == "PAIR+NLIST":
                pairs = orc.nl_classic(m, n0, n1, pos, TRIC_BOX, True, 1.1)
        else:
            pairs = orc.all_pairs(m, n0, n1)
        if nl and (step % 2 == 0 or kind == "PAIR+NLIST"):
            assert np.array_equal(_sorted(c.pairs()), _sorted(pairs)), step
        _check("mixed", got, orc.coordination(spec, pos, TRIC_BOX, pairs), "%s step %d" % (kind, step))
        pos = pos + rng.normal(0.0, 0.01, pos.shape)
    c.close()


@pytest.mark.parametrize("spec", ["RATIONAL R_0=0.3 NN=6 MM=12", "EXP R_0=0.2 D_0=0.1",
                                  "CUSTOM FUNC=1/(1+x^6) R_0=0.3 D_MAX=0.7"])
def test_mixed_triclinic_small_box_shifts(orc, spec):
    """A 1.5 nm triclinic box and no (or a long) D_MAX: distant pairs take the
    octant shifts of Pbc::distance."""
    from plumed2_gb300.action import Coordination
    box = TRIC_BOX / 2.0
    pos = _tric_frame(5, box, 0.02, 4)
    c = Coordination("GROUPA=1-125 SWITCH={%s}" % spec, precision="mixed")
    got = c.calculate(pos, box)
    _check("mixed", got, orc.coordination(spec, pos, box, orc.all_pairs(0, 125)), spec)


@pytest.mark.parametrize("m,a,kind", [(5, 0.25, "NLIST"), (5, 0.3, "NLISTCELLS"), (8, 0.25, "NLIST"),
                                       (8, 0.3, "NLIST"), (16, 0.25, "NLIST"), (16, 0.3, "NLISTCELLS"),
                                       (10, 0.25, "none")])
def test_mixed_dmax_band_on_a_lattice(orc, m, a, kind):
    """A perfect simple-cubic lattice whose spacing is D_MAX: every
    nearest-neighbour pair lies in the FP32 band around D_MAX^2 and is decided
    by the FP64 fix-up (3 m^3 such pairs: 375 fit the frame's queue, 1,536
    and 12,288 take the flagged-slice rescan; 0.25 is exact in binary, so
    those pairs are all in, 0.3 is not).  Values and the pair set against the oracle over two calls
    (the fix-up resets its queue)."""
    from plumed2_gb300.action import Coordination
    from plumed2_gb300.frames import sc_sites
    n = m ** 3
    pos = sc_sites(n) * a
    box = np.diag([m * a] * 3)
    spec = "RATIONAL R_0=%.2f NN=6 MM=12 D_MAX=%.2f NOSTRETCH" % (0.8 * a, a)  # nonzero at D_MAX
    nl = "" if kind == "none" else " %s NL_CUTOFF=%.2f NL_STRIDE=1" % (kind, 1.5 * a)
    c = Coordination("GROUPA=1-%d SWITCH={%s}%s" % (n, spec, nl), precision="mixed")
    for step in range(2):
        got = c.calculate(pos, box, step)
        if kind == "none":
            pairs = orc.all_pairs(0, n)
        else:
            pairs = (orc.nl_classic if kind == "NLIST" else orc.nl_linkcells)(0, n, 0, pos, box, True, 1.5 * a)
            assert np.array_equal(_sorted(c.pairs()), _sorted(pairs))
        ref = orc.coordination(spec, pos, box, pairs)
        _check("mixed", got, ref, "step %d" % step, dfloor=np.abs(ref[2]).max())
    c.close()


def test_rt20_switch_goldens(golden):
    """regtest/basic/rt20-switch-*: two atoms over switchtraj.xyz through the GPU."""
    from plumed2_gb300.action import Coordination
    g = golden("rt20_switch.json")
    for name, case in g["cases"].items():
        colvar = np.array(case["colvar"])
        deriv = np.array(case["deriv"])
        cc = {lab: Coordination("GROUPA=1 GROUPB=2 SWITCH={%s}" % case[lab]) for lab in ("c", "cs")}
        for fi, (frame, box) in enumerate(zip(g["traj"], g["box"])):
            B = np.diag(box)
            for col, lab in ((1, "c"), (2, "cs")):
                s, d, v = cc[lab].calculate(np.array(frame), B)
                assert abs(s - colvar[fi, col]) <= 5.01e-7, (name, lab, fi)
                rows = deriv[deriv[:, 0] == colvar[fi, 0]]
                got = np.concatenate([d.reshape(-1), v.reshape(-1)])
                assert np.all(np.abs(got - rows[:, 1 + col]) <= 5.01e-5), (name, lab, fi)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["NLIST", "NLISTCELLS"])
@pytest.mark.parametrize("groups", ["GROUPA=8853-8937", "GROUPA=8001-8333 GROUPB=8500-8700", "GROUPA=1-1000"])
def test_nlist_ragged_slices(orc, prec, kind, groups):
    """Group sizes that are not a multiple of 32 (a partial last slice of the
    neighbour list), taken as clustered sub-ranges of a larger lattice."""
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.436 NN=6 MM=12 D_MAX=1.0"
    n, L = 12167, 23 * 0.31
    box = np.diag([L] * 3)
    full = jittered_lattice(n, 0.31, 0.03, 200)
    c = Coordination("%s SWITCH={%s} %s NL_CUTOFF=1.2 NL_STRIDE=5" % (groups, spec, kind), precision=prec)
    pos = full[c.requested_atoms]
    nA = c.nslots if "GROUPB" not in groups else 333
    m, n0, n1 = (0, c.nslots, 0) if "GROUPB" not in groups else (1, nA, c.nslots - nA)
    got = c.calculate(pos, box, 0)
    if kind == "NLIST":
        ref_pairs = orc.nl_classic_cells(m, n0, n1, pos, box, True, 1.2)
    else:
        ref_pairs = orc.nl_linkcells(m, n0, n1, pos, box, True, 1.2)
    assert np.array_equal(_sorted(c.pairs()), _sorted(ref_pairs))
    ref = orc.coordination(spec, pos, box, ref_pairs)
    _check(prec, got, ref, groups)
    c.close()


def test_empty_and_tiny_groups(orc):
    from plumed2_gb300.action import Coordination
    box = np.diag([3.0] * 3)
    c = Coordination("GROUPA=1 GROUPB=1 R_0=0.3")  # the self pair is skipped: 0
    s, d, v = c.calculate(np.zeros((2, 3)), box)
    assert s == 0.0 and np.all(d == 0)
    c = Coordination("GROUPA=1-2 R_0=0.3")
    pos = np.array([[0.0, 0, 0], [0.25, 0, 0]])
    s, d, v = c.calculate(pos, box)
    ref = orc.coordination("R0SYNTAX 6 0 0.3 0.0", pos, box, np.array([[0, 1]], np.uint32))
    _check("fp64", (s, d, v), ref)


def test_walkers_batched_device(orc):
    """Several walkers in one launch (coord_forward_device), each with its own list."""
    torch = pytest.importorskip("torch")
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.6"
    n, L, W = 4096, 16 * 0.31, 3
    box = np.diag([L] * 3)
    frames = np.stack([jittered_lattice(n, 0.31, 0.03, 100 + w) for w in range(W)])
    for prec in ("fp64", "mixed"):
        c = Coordination("GROUPA=1-4096 SWITCH={%s} NLIST NL_CUTOFF=0.8 NL_STRIDE=10" % spec, precision=prec)
        dev = torch.device("cuda:0")
        tpos = torch.from_numpy(frames).to(dev)
        s = torch.zeros(W, dtype=torch.float64, device=dev)
        der = torch.zeros(W, n, 3, dtype=torch.float64, device=dev)
        vir = torch.zeros(W, 9, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        c.forward_device(tpos.data_ptr(), np.stack([box] * W), W, s.data_ptr(), der.data_ptr(), vir.data_ptr(),
                         step=0)
        torch.cuda.synchronize()
        for w in range(W):
            pairs = orc.nl_classic_cells(0, n, 0, frames[w], box, True, 0.8)
            assert np.array_equal(_sorted(c.pairs(w)), pairs)
            ref = orc.coordination(spec, frames[w], box, pairs)
            _check(prec, (s[w].item(), der[w].cpu().numpy(), vir[w].cpu().numpy().reshape(3, 3)), ref, prec)


def test_mixed_flat_slab_far_apart_ranks(orc):
    """A flat periodic slab (99 x 20 x 3 cells, about 106k atoms): partners in
    the neighbouring cell layer lie more than 32,767 ranks away, and two of
    the three z cells wrap.  Pair set bit-exact, values within the mixed
    tolerance, also on the step that reuses the list."""
    from plumed2_gb300.action import Coordination
    nx, ny, nz, a0 = 256, 52, 8, 0.31
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    sites = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1) * a0
    pos = sites + np.random.default_rng(8).normal(0.0, 0.03, sites.shape)
    box = np.diag([nx * a0, ny * a0, nz * a0])
    n = len(pos)
    spec = "RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.6"
    c = Coordination("GROUPA=1-%d SWITCH={%s} NLIST NL_CUTOFF=0.8 NL_STRIDE=10" % (n, spec), precision="mixed")
    got = c.calculate(pos, box, 0)
    pairs = orc.nl_classic_cells(0, n, 0, pos, box, True, 0.8)
    assert np.array_equal(_sorted(c.pairs()), pairs)
    ref = orc.coordination(spec, pos, box, pairs, nthreads=orc.max_threads())
    _check("mixed", got, ref)
    got = c.calculate(pos + 0.01, box, 1)  # the same list, without a rebuild
    ref = orc.coordination(spec, pos + 0.01, box, pairs, nthreads=orc.max_threads())
    _check("mixed", got, ref)
