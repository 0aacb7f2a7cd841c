"""The PLUMED plugin's own C++ code on the GPU: CoordinationGPU.cpp compiled
unchanged against the harness's minimal action interface (tests/plugin_host)
and stepped through frames as `plumed driver` steps an action -- prepare(),
then the requested atoms, then calculate().  Per frame: the value, the
derivatives by atom number and the box derivatives against the C oracle on
the same frames.

The neighbour-list cases exercise NeighborList::prepare's request cycle in the
plugin (NeighborList.cpp:317-355, 433-456): the full request on rebuild steps
(multiples of NL_STRIDE), only the atoms of the list in between, with the
derivatives then mapped back through the reduced list.  Tolerances: FP64
|ds|/s <= 1e-12, derivatives and virial <= 1e-11 of their scale; MIXED 1e-6
and 1e-5.  The list is the one built at the last rebuild step."""
import numpy as np
import pytest

from plumed2_gb300.frames import jittered_lattice
from tests.plugin_host import harness

pytestmark = pytest.mark.gpu

TOL = {"FP64": (1e-12, 1e-11), "MIXED": (1e-6, 1e-5)}


def _trajectory(n, a, steps, seed, step_sigma):
    rng = np.random.default_rng(seed)
    x = jittered_lattice(n, a, 0.03, seed)
    out = [x]
    for _ in range(steps - 1):
        out.append(out[-1] + rng.normal(0.0, step_sigma, size=x.shape))
    return np.stack(out)


def _oracle(orc, spec, ga, gb, frames, box, nl=None, stride=1, pair=False):
    """s, derivatives by atom, virial and requested-atom count per frame, as the
    reference's action computes them (NLIST: classic list at the steps that
    are multiples of NL_STRIDE, reduced request in between)."""
    absi = np.array(list(ga) + list(gb))
    mode = 2 if pair else (1 if len(gb) else 0)
    n0, n1 = len(ga), len(gb)
    out, pairs = [], None
    for k, x in enumerate(frames):
        pos = x[absi]
        step = k
        if nl is None:
            if pairs is None:
                pairs = orc.all_pairs(mode, n0, n1)
            req = len(absi)
        else:
            rebuild = pairs is None or stride <= 1 or step % stride == 0
            if rebuild:
                # NLIST: the classic list; NLISTCELLS: every pair of neighbouring link cells
                pairs = (orc.nl_linkcells if nl[1] else orc.nl_classic)(mode, n0, n1, pos, box, True, nl[0])
                req = len(absi)
            else:
                req = len(np.unique(absi[pairs.reshape(-1)])) if stride > 1 else len(absi)
        s, d, v = orc.coordination(spec, pos, box, pairs, abs_index=absi, nthreads=orc.max_threads())
        D = np.zeros_like(x)
        np.add.at(D, absi, d)
        out.append((s, D, v, req))
    return out


def _check(prec, got, ref, what):
    vals, der, vir, nreq, _ = got
    ts, td = TOL[prec]
    for k, (s0, d0, v0, r0) in enumerate(ref):
        assert abs(vals[k] - s0) <= ts * abs(s0), (what, k, vals[k], s0)
        sc = np.abs(d0).max()
        assert np.abs(der[k] - d0).max() <= td * sc, (what, k, np.abs(der[k] - d0).max() / sc)
        assert np.abs(vir[k] - v0).max() <= td * np.abs(v0).max(), (what, k)
        assert nreq[k] == r0, (what, k, nreq[k], r0)


@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
def test_plugin_every_pair(orc, prec):
    from plumed2_gb300 import frames as W
    spec = "RATIONAL R_0=0.30 D_0=0.0 NN=6 MM=12 D_MAX=1.0"
    xs = np.stack([W.workload_c0(frame=f)[0] for f in range(3)])
    box = W.workload_c0()[1]
    got = harness.run("c: COORDINATION GROUPA=1-1000 SWITCH={%s} PRECISION=%s" % (spec, prec), xs, [box] * 3)
    _check(prec, got, _oracle(orc, spec, range(1000), [], xs, box), "C0 " + prec)


@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
@pytest.mark.parametrize("cells", [False, True])
def test_plugin_neighbour_list_request_cycle(orc, prec, cells):
    """12 frames moving by 0.01 nm Gaussian steps, NL_STRIDE=5: rebuilds at
    steps 0, 5, 10; reduced requests on the others (pairs that were within the
    cutoff at the rebuild keep being evaluated as they move)."""
    n, a = 2744, 0.31
    L = 14 * a
    xs = _trajectory(n, a, 12, 31, 0.01)
    box = np.diag([L] * 3)
    spec = "RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.7"
    kw = "NLISTCELLS" if cells else "NLIST"
    line = ("c: COORDINATION GROUPA=1-1500 GROUPB=1201-2744 SWITCH={%s} %s NL_CUTOFF=0.8 NL_STRIDE=5 PRECISION=%s"
            % (spec, kw, prec))
    got = harness.run(line, xs, [box] * len(xs))
    ref = _oracle(orc, spec, range(1500), range(1200, 2744), xs, box, nl=(0.8, cells), stride=5)
    _check(prec, got, ref, line)
    # the reduced request is smaller than the full one on the steps between rebuilds
    assert all(got[3][k] < 1500 + 1544 for k in range(12) if k % 5)


def test_plugin_pair_and_overlapping_groups(orc):
    """PAIR (NeighborList.cpp:150-152) and groups sharing atoms, FP64."""
    xs = _trajectory(1000, 0.3, 3, 7, 0.01)
    box = np.diag([3.0] * 3)
    spec = "RATIONAL R_0=0.3 NN=6 MM=12 D_MAX=1.2"
    got = harness.run("c: COORDINATION GROUPA=1-400 GROUPB=301-700 SWITCH={%s} PAIR" % spec, xs, [box] * 3)
    _check("FP64", got, _oracle(orc, spec, range(400), range(300, 700), xs, box, pair=True), "PAIR")
    got = harness.run("c: COORDINATION GROUPA=1-10 GROUPB=30-40,5,50-100 SWITCH={%s}" % spec, xs, [box] * 3)
    gb = list(range(29, 40)) + [4] + list(range(49, 100))
    _check("FP64", got, _oracle(orc, spec, range(10), gb, xs, box), "overlapping groups")
