"""The C oracle is bit-identical to the reference's own code on the same inputs.

Runs where oracle/_ref (the reference sources compiled by oracle/Makefile)
exists; skipped elsewhere.  Serial order and -ffp-contract=off on both sides
make every comparison exact (np.array_equal), not toleranced, except for
CUSTOM switching functions: the reference differentiates the lepton
expression symbolically and simplifies it, the oracle differentiates it
forward, so those agree within 1e-13 relative (most results bit for bit).
"""
import numpy as np
import pytest

from plumed2_gb300.frames import jittered_lattice

SPECS = [
    "RATIONAL R_0=0.30 D_0=0.0 NN=6 MM=12 D_MAX=1.0",
    "RATIONAL R_0=1.3 NN=6 MM=10 D_MAX=2.6",
    "RATIONAL R_0=1.3 NN=5 MM=11 D_MAX=2.6",
    "RATIONAL R_0=1.3 NN=5 D_MAX=2.6",
    "RATIONAL R_0=0.3 NN=8 MM=16 D_MAX=0.9",
    "RATIONAL R_0=0.3 NN=6 MM=12",
    "RATIONAL R_0=1.3 NN=6 MM=10 D_MAX=2.6 NOSTRETCH",
    "EXP R_0=0.8 D_0=0.5 D_MAX=2.6",
    "GAUSSIAN R_0=1.0 D_0=0.0 D_MAX=2.6",
    "GAUSSIAN R_0=1.0 D_0=0.3 D_MAX=2.6",
    "Q R_0=1.0 D_0=0.3 BETA=5.0 LAMBDA=1.0 REF=1.3 D_MAX=2.6",
    "TANH R_0=1.3 D_MAX=2.6",
    "SMAP R_0=1.3 A=3 B=2 D_MAX=2.6",
    "CUBIC D_MAX=2.6 D_0=0.6",
    "COSINUS R_0=2.6",
    "R0SYNTAX 6 0 0.3 0.0",
    "R0SYNTAX 7 0 1.0 0.1",
    "R0SYNTAX 8 14 0.4 0.05",
]


@pytest.mark.parametrize("spec", SPECS)
def test_switch_bit_exact(orc, ref, spec):
    x = np.linspace(0.0, 3.0, 3001)
    for squared in (True, False):
        xx = x * x if squared else x
        f1, d1 = orc.switch_eval(spec, xx, squared)
        f2, d2 = ref.switch_eval(spec, xx, squared)
        assert np.array_equal(f1, f2) and np.array_equal(d1, d2)


def test_pbc_bit_exact(orc, ref):
    rng = np.random.default_rng(11)
    for box in (np.diag([3.0, 3.1, 2.9]),
                np.array([[3, 0, 0], [0.5, 2.8, 0], [0.3, 0.2, 2.9]], float),
                np.array([[6, -6, 0], [0, 6, -6], [-6, 6, 6]], float),
                np.zeros((3, 3))):
        v1 = rng.uniform(-5, 5, (400, 3))
        v2 = rng.uniform(-5, 5, (400, 3))
        d2, _ = ref.pbc_distance(box, v1, v2)
        assert np.array_equal(orc.pbc_distance(box, v1, v2), d2)


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("do_pbc", [True, False])
def test_neighbour_list_bit_exact(orc, ref, mode, do_pbc):
    pos = jittered_lattice(1000, 0.30, 0.03, 5)
    box = np.diag([3.0] * 3)
    n0, n1 = (1000, 0) if mode == 0 else (500, 500)
    for cut in (0.45, 0.9, 1.6):
        a = orc.nl_classic(mode, n0, n1, pos, box, do_pbc, cut)
        b = ref.nl(mode, n0, n1, pos, box, do_pbc, cut)
        assert np.array_equal(a, b)
        if mode != 2:
            c = orc.nl_linkcells(mode, n0, n1, pos, box, do_pbc, cut)
            d = ref.nl(mode, n0, n1, pos, box, do_pbc, cut, cells=True)
            assert np.array_equal(c, d)


@pytest.mark.parametrize("spec", ["RATIONAL R_0=0.30 D_0=0.0 NN=6 MM=12 D_MAX=1.0", "R0SYNTAX 6 0 0.3 0.0",
                                  "RATIONAL R_0=0.3 NN=5 MM=11 D_MAX=1.0", "GAUSSIAN R_0=0.2 D_0=0.1 D_MAX=0.9"])
def test_coordination_bit_exact(orc, ref, spec):
    pos = jittered_lattice(1000, 0.30, 0.03, 6)
    box = np.diag([3.0] * 3)
    for mode, n0, n1, cut in ((0, 1000, 0, 0.0), (0, 1000, 0, 0.8), (1, 400, 600, 0.0), (1, 400, 600, 0.9),
                              (2, 500, 500, 0.0)):
        s2, d2, v2 = ref.coordination(spec, mode, n0, n1, pos, box, nl_cutoff=cut)
        pairs = orc.all_pairs(mode, n0, n1) if cut == 0 else orc.nl_classic(mode, n0, n1, pos, box, True, cut)
        s1, d1, v1 = orc.coordination(spec, pos, box, pairs)
        assert s1 == s2 and np.array_equal(d1, d2) and np.array_equal(v1, v2)


def test_coordination_duplicates_and_self_skip(orc, ref):
    """GROUPA with repeated atoms (cf. regtest/basic/rt-fix-229): pairs of equal absolute index are skipped."""
    pos0 = jittered_lattice(64, 0.3, 0.03, 8)
    sel = np.array([0, 1, 1, 2, 5, 5, 5, 9, 30, 31, 63, 0])
    pos = pos0[sel]
    box = np.diag([1.2] * 3)
    spec = "R0SYNTAX 6 0 0.3 0.0"
    s2, d2, v2 = ref.coordination(spec, 0, len(sel), 0, pos, box, abs_index=sel.astype(np.int64))
    s1, d1, v1 = orc.coordination(spec, pos, box, orc.all_pairs(0, len(sel)), abs_index=sel)
    assert s1 == s2 and np.array_equal(d1, d2) and np.array_equal(v1, v2)


def test_linkcells_required_cells(orc, ref):
    """Link-cell counts and the cells searched from a cell, with and without
    PBC, against the reference's LinkCells (setupCells(pbc) and
    addRequiredCells): orthorhombic, flat and skewed boxes, cutoffs from
    below one cell up to a third of the box, every kind of cell.  Boxes
    with their rows permuted into a left-handed order have a negative
    volume, and both refuse them, for the cells and for the list."""
    rng = np.random.default_rng(12)
    n = 0
    for _ in range(300):
        kind = rng.integers(0, 3)
        if kind == 0:
            box = np.diag(rng.uniform(1.0, 10.0, 3))
        elif kind == 1:
            box = np.diag([rng.uniform(0.5, 2.0), rng.uniform(4.0, 10.0), rng.uniform(4.0, 10.0)])[rng.permutation(3)]
        else:
            box = rng.uniform(-1.0, 1.0, (3, 3)) * 3.0 + np.eye(3) * 6.0
        cut = rng.uniform(0.15, 0.5) * min(np.abs(np.linalg.det(box)) ** (1 / 3), 6.0)
        if np.linalg.det(box) <= 0:  # left-handed: both refuse it (LinkCells.cpp:81)
            with pytest.raises(ValueError, match="null volume"):
                ref.linkcells_required(box, cut, [0, 0, 0])
            pos = rng.random((40, 3)) @ box
            with pytest.raises(ValueError, match="null volume"):
                orc.nl_linkcells(0, 40, 0, pos, box, True, cut)
            with pytest.raises(ValueError, match="refused"):
                ref.nl(0, 40, 0, pos, box, True, cut, cells=True)
            n += 2
            continue
        lim = orc.linkcells_ncells(box, cut)
        cell = [int(rng.integers(0, lim[k])) for k in range(3)]
        for use_pbc in (True, False):
            rlim, rreq = ref.linkcells_required(box, cut, cell, use_pbc)
            assert lim == rlim, (box, cut)
            assert orc.linkcells_required(box, cut, cell, use_pbc) == rreq, (box, cut, cell, use_pbc)
            n += 1
    assert n == 600


CUSTOM_FUNCS = [
    "1/(1+x^6)", "(1+x^3)/(1+x^9)", "exp(-x)", "exp(-0.5*x^2)", "1/(1+x2^3)", "exp(-x2/2)",
    "step(x)*0.5*(cos(x*pi)+1)+step(-x)*1.0", "1-tanh(x)", "erfc(x)", "1/(1+exp(10*(x-1)))",
    "select(step(1-x),1-x^2,0)", "max(0,1-x)^2", "min(1,1/x^3)", "abs(x-1.3)*exp(-x)", "sqrt(1+x)^-3",
    "x^x*exp(-3*x)", "atan2(1,x)/pi", "(cos(pi*x)+1)/2*step(1-x)", "cube(1-x)*step(1-x)", "recip(1+square(x))",
    "log(1+exp(-x))", "1/cosh(x)^2", "-x^2+1", "2^-x", "ceil(3-x)/3*exp(-x)", "sinh(x)/cosh(x)", "1/(1+x^2.5)",
    "2*pi*exp(-x)/(2*pi)", "1e-1*x^-2/(1+1e-1*x^-2)", "sec(x/4)-csc(1+x)*sin(1+x)", "cot(1+x)*tan(1+x)*exp(-x)",
    "asin(1/(1+x))+acos(1/(1+x))-pi_2+exp(-x)"]


def _close(a, b, tol):
    a, b = np.asarray(a), np.asarray(b)
    same = (a == b) | (np.abs(a - b) <= tol * np.maximum(np.abs(b), 1e-300)) | (np.isnan(a) & np.isnan(b))
    return bool(np.all(same))


@pytest.mark.parametrize("func", CUSTOM_FUNCS)
def test_custom_switch(orc, ref, func):
    """CUSTOM (lepton) switching functions of x and x2, with D_0, D_MAX and
    NOSTRETCH, against the reference's leptonSwitch, both calculate and
    calculateSqr, across and beyond D_MAX."""
    x = np.concatenate([np.linspace(0.01, 3.0, 300), [0.1, 0.2, 1.0]])
    for extra in ("R_0=0.7", "R_0=1.1 D_0=0.2", "R_0=0.9 D_MAX=2.5", "R_0=0.5 D_0=0.1 D_MAX=1.9 NOSTRETCH"):
        spec = "CUSTOM FUNC=%s %s" % (func, extra)
        for squared in (True, False):
            xx = x * x if squared else x
            f1, d1 = orc.switch_eval(spec, xx, squared)
            f2, d2 = ref.switch_eval(spec, xx, squared)
            assert _close(f1, f2, 1e-13) and _close(d1, d2, 1e-13), spec


def test_custom_switch_refusals(orc, ref):
    """Two variables, a name other than x or x2, an unknown function: both
    refuse, with the reference's messages for the first two kinds."""
    x = np.array([0.5])
    for func in ("x*x2", "y+x", "foo(x)"):
        spec = "CUSTOM FUNC=%s R_0=1" % func
        with pytest.raises(ValueError):
            ref.switch_eval(spec, x)
        with pytest.raises(ValueError) as e:
            orc.switch_eval(spec, x)
        want = ("unknown function: foo" if func == "foo(x)" else
                "Please declare a function with only ONE argument that can only be x or x2")
        assert want in str(e.value)


def test_coordination_custom_switch(orc, ref):
    """The CV with a CUSTOM switch (regtest/basic/rt42's d) on single, two-list
    and PAIR groups, with and without a list."""
    pos = jittered_lattice(1000, 0.30, 0.03, 6)
    box = np.diag([3.0] * 3)
    for spec in ("CUSTOM FUNC=1/(1+x^6) R_0=0.3 D_MAX=1.0", "CUSTOM FUNC=exp(-x2/2) R_0=0.25 D_MAX=0.9"):
        for mode, n0, n1, cut in ((0, 1000, 0, 0.0), (0, 1000, 0, 1.1), (1, 400, 600, 0.0), (2, 500, 500, 0.0)):
            s2, d2, v2 = ref.coordination(spec, mode, n0, n1, pos, box, nl_cutoff=cut)
            pairs = orc.all_pairs(mode, n0, n1) if cut == 0 else orc.nl_classic(mode, n0, n1, pos, box, True, cut)
            s1, d1, v1 = orc.coordination(spec, pos, box, pairs)
            assert abs(s1 - s2) <= 1e-13 * abs(s2)
            assert np.abs(d1 - d2).max() <= 1e-12 * np.abs(d2).max()
            assert np.abs(v1 - v2).max() <= 1e-12 * np.abs(v2).max()


@pytest.mark.parametrize("func", CUSTOM_FUNCS)
def test_library_custom_switch_host_values(orc, ref, func):
    """The library's own CUSTOM compiler and evaluator (host side, the code the
    kernels run) against the reference's leptonSwitch and the oracle, both
    calculate and calculateSqr, across and beyond D_MAX: within 1e-12
    relative (the reference differentiates symbolically and simplifies)."""
    from plumed2_gb300.action import Coordination
    x = np.concatenate([np.linspace(0.01, 3.0, 300), [0.1, 0.2, 1.0]])
    for extra in ("R_0=0.7", "R_0=1.1 D_0=0.2", "R_0=0.9 D_MAX=2.5", "R_0=0.5 D_0=0.1 D_MAX=1.9 NOSTRETCH"):
        spec = "CUSTOM FUNC=%s %s" % (func, extra)
        c = Coordination("GROUPA=1-2 SWITCH={%s}" % spec)
        for squared in (True, False):
            xx = x * x if squared else x
            f, d = c.switch(xx, squared)
            fr, dr = ref.switch_eval(spec, xx, squared)
            fo, do = orc.switch_eval(spec, xx, squared)
            assert _close(f, fr, 1e-12) and _close(d, dr, 1e-12), (spec, squared)
            assert _close(f, fo, 1e-12) and _close(d, do, 1e-12), (spec, squared)
        c.close()
