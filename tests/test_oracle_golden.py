"""The C oracle against the reference's own regtest golden outputs.

Every expected number here was printed by the reference (regtest
``*.reference`` files, extracted by tests/golden/make_golden.py); the
tolerance is the rounding of the print format that produced it.
"""
import numpy as np
import pytest

from plumed2_gb300.frames import sc_sites


def test_rt_make_switch(orc, golden):
    """regtest/basic/rt-make-switch: value and derivative at 10 points, %.6f."""
    g = golden("rt_make_switch.json")
    assert len(g["cases"]) == 24
    for name, case in g["cases"].items():
        rows = np.array(case["rows"])
        f, df = orc.switch_eval(case["definition"], rows[:, 0], squared=False)
        assert np.all(np.abs(f - rows[:, 1]) <= 5.01e-7), name
        assert np.all(np.abs(df - rows[:, 2]) <= 5.01e-7), name
        # calculateSqr agrees with calculate to the printed precision (the
        # vsq_delta columns of the same file are all +-0.000000)
        f2, df2 = orc.switch_eval(case["definition"], rows[:, 0] ** 2, squared=True)
        assert np.all(np.abs(f2 - f) <= 5e-7) and np.all(np.abs(df2 - df) <= 5e-7), name


def _two_atom_cv(orc, spec, a, b, box):
    pos = np.array([a, b], float)
    return orc.coordination(spec, pos, box, np.array([[0, 1]], np.uint32))


def test_rt20_switch(orc, golden):
    """regtest/basic/rt20-switch-*: COLVAR (%f) and DUMPDERIVATIVES (%8.4f)."""
    g = golden("rt20_switch.json")
    assert len(g["cases"]) == 12
    for name, case in g["cases"].items():
        colvar = np.array(case["colvar"])
        deriv = np.array(case["deriv"])
        for fi, (frame, box) in enumerate(zip(g["traj"], g["box"])):
            B = np.diag(box) if len(box) == 3 else np.array(box).reshape(3, 3)
            for col, lab in ((1, "c"), (2, "cs")):
                s, d, v = _two_atom_cv(orc, case[lab], frame[0], frame[1], B)
                assert abs(s - colvar[fi, col]) <= 5.01e-7, (name, lab, fi)
                rows = deriv[deriv[:, 0] == colvar[fi, 0]]
                got = np.concatenate([d.reshape(-1), v.reshape(-1)])
                assert np.all(np.abs(got - rows[:, 1 + col]) <= 5.01e-5), (name, lab, fi)


def test_rt42_values_forces_virial(orc, golden):
    """regtest/basic/rt42 (+rt42c): 108 atoms in a triclinic box.

    c, e, g at %8.4f; forces and full virial of RESTRAINT SLOPE=1 on c+d (plus
    the SLOPE=0.001 restraint on the CUSTOM cross-check combination
    c - d/2 - dfast/2 + e - f + g - h) at %10.5f, with d, dfast, f and h the
    regtest's own CUSTOM (lepton) definitions.
    """
    g = golden("rt42.json")
    for fi in range(len(g["frames"])):
        pos = np.array(g["frames"][fi])
        box = np.array(g["box"][fi]).reshape(3, 3)
        n = len(pos)
        pos2 = np.concatenate([pos, pos])
        absi = np.concatenate([np.arange(n), np.arange(n)])
        pairs = orc.all_pairs(1, n, n)

        def cv(spec):
            s, d, v = orc.coordination(spec, pos2, box, pairs, abs_index=absi)
            return s, d[:n] + d[n:], v

        sc, dc, vc = cv("R0SYNTAX 6 0 1.0 0.0")
        sd, dd, vd = cv("CUSTOM FUNC=1/(1+x^6) R_0=1")
        _, dq, vq = cv("CUSTOM FUNC=1/(1+x2^3) R_0=1")
        se, de, ve = cv("R0SYNTAX 7 0 1.0 0.1")
        sf, df, vf = cv("CUSTOM FUNC=1/(1+x^7) R_0=1 D_0=0.1")
        sg, dg, vg = cv("EXP R_0=1")
        _, dh, vh = cv("CUSTOM FUNC=exp(-x) R_0=1")
        s1, _, _ = orc.coordination("R0SYNTAX 6 0 1.0 0.0", pos, box, orc.all_pairs(0, n))
        assert abs(sc - g["c"][fi]) <= 5.01e-5
        assert abs(se - g["e"][fi]) <= 5.01e-5
        assert abs(sg - g["g"][fi]) <= 5.01e-5
        assert abs(s1 - g["c_single"][fi]) <= 5.01e-5
        F = -(dc + dd) - 0.001 * (dc - 0.5 * dd - 0.5 * dq + de - df + dg - dh)
        V = -(vc + vd) - 0.001 * (vc - 0.5 * vd - 0.5 * vq + ve - vf + vg - vh)
        assert np.abs(F - np.array(g["ff_forces"][fi])).max() <= 5.01e-6
        assert np.abs(V - np.array(g["ff_virial"][fi]).reshape(3, 3)).max() <= 5.01e-6


def test_rt42b_gro_triclinic(orc, golden):
    """regtest/basic/rt42b: GROUPA=GROUPB=1-108 R_0=1 (each pair twice, self
    pairs skipped) over a .gro trajectory with triclinic boxes, %8.4f."""
    g = golden("rt42b.json")
    n = 108
    absi = np.concatenate([np.arange(n), np.arange(n)])
    pairs = orc.all_pairs(1, n, n)
    for fi, (fr, bx) in enumerate(zip(g["frames"], g["box"])):
        pos = np.array(fr)[absi]
        s, _, _ = orc.coordination("R0SYNTAX 6 0 1 0.0", pos, np.array(bx).reshape(3, 3), pairs, abs_index=absi)
        assert abs(s - g["c"][fi]) <= 5.01e-5, fi


def test_rt_mpi0_overlapping_groups(orc, golden):
    """regtest/basic/rt-mpi0: GROUPA=1-10, GROUPB=30-40,5,50-100 (atom 5 in
    both: its self pair is skipped, and it has a derivative entry in each
    group).  c, cexp, cgaus (%6.3f); DUMPDERIVATIVES of cexp and cgaus, 3 per
    requested atom then the box (%8.4f); forces and virial diagonal of
    RESTRAINT KAPPA=5 AT=15 on c (%f)."""
    from plumed2_gb300.action import parse_atom_list
    g = golden("rt_mpi0.json")
    ga, gb = parse_atom_list(g["groupa"]), parse_atom_list(g["groupb"])
    absi = np.array(ga + gb)
    pairs = orc.all_pairs(1, len(ga), len(gb))
    rs = g["restraint"]
    for fi, (fr, bx) in enumerate(zip(g["frames"], g["box"])):
        frame = np.array(fr)
        pos = frame[absi]
        box = np.diag(bx) if len(bx) == 3 else np.array(bx).reshape(3, 3)
        res = {k: orc.coordination(spec, pos, box, pairs, abs_index=absi) for k, spec in g["switch"].items()}
        for k in ("c", "cexp", "cgaus"):
            assert abs(res[k][0] - g["colvar"][fi][k]) <= 5.01e-4, (fi, k)
        for k in ("cexp", "cgaus"):
            got = np.concatenate([res[k][1].reshape(-1), res[k][2].reshape(-1)])
            assert np.abs(got - np.array(g["deriv_" + k][fi])).max() <= 5.01e-5, (fi, k)
        s, d, v = res[rs["arg"]]
        w = -rs["kappa"] * (s - rs["at"])
        F = np.zeros_like(frame)
        np.add.at(F, absi, w * d)
        assert np.abs(F - np.array(g["ff_forces"][fi])).max() <= 5.01e-7, fi
        assert np.abs(w * np.diag(v) - np.array(g["ff_virial_diag"][fi])).max() <= 5.01e-7, fi


def _rt42_cells_steps(orc, g, spec):
    """The two CVs of an rt42-cells input over its trajectory, lists rebuilt
    on steps that are multiples of NL_STRIDE=4: (s, derivatives per atom,
    virial) of the NLIST one (c) and of the NLISTCELLS one (d) per step."""
    n = len(g["frames"][0])
    absi = np.concatenate([np.arange(n), np.arange(n)])
    out = []
    for step, (fr, bx) in enumerate(zip(g["frames"], g["box"])):
        pos = np.array(fr)
        box = np.array(bx).reshape(3, 3)
        pos2 = np.concatenate([pos, pos])
        if step % 4 == 0:
            pc = orc.nl_classic(1, n, n, pos2, box, True, 2.0)
            pd = orc.nl_linkcells(1, n, n, pos2, box, True, 2.0)
        res = []
        for pairs in (pc, pd):
            s, d, v = orc.coordination(spec, pos2, box, pairs, abs_index=absi)
            res.append((s, d[:n] + d[n:], v))
        out.append(res)
    return out


@pytest.mark.parametrize("variant", ["rt42-cells", "rt42-cells-cos", "rt42-cells-gauss"])
def test_rt42_cells_nlist_vs_nlistcells(orc, golden, variant):
    """regtest/basic/rt42-cells{,-cos,-gauss}: GROUPA=GROUPB=1-108 in a
    triclinic box, NLIST against NLISTCELLS with D_MAX (or the COSINUS cutoff)
    below NL_CUTOFF.  d - c at %8.4f (check_diff.reference) and the forces and
    virial of RESTRAINT SLOPE=0.001 on d - c at %10.5f (ff.reference) are zero
    on every one of the 27 frames."""
    import re
    g = golden("rt42_cells.json")
    v = g["variants"][variant]
    spec = re.search(r"SWITCH=\{([^}]*)\}", v["c"]).group(1).strip()
    assert v["ff_max_abs"] == 0.0
    for step, ((sc, dc, vc), (sd, dd, vd)) in enumerate(_rt42_cells_steps(orc, g, spec)):
        assert abs((sd - sc) - v["check_diff"][step]) <= 5.01e-5, step
        assert np.abs(0.001 * (dd - dc)).max() <= 5.01e-6, step
        assert np.abs(0.001 * (vd - vc)).max() <= 5.01e-6, step
        assert sc > 0


def _neigh_sets(pairs, nslots):
    out = [set() for _ in range(nslots)]
    for a, b in pairs:
        out[a].add(int(b))
        out[b].add(int(a))
    return out


@pytest.mark.parametrize("pbc", ["off", "on"])
def test_rt_neighbourlist(orc, golden, pbc):
    """regtest/tools/rt-Neigbourlist: exact neighbour sets (sc lattice, cutoff 1.999 spacing)."""
    g = golden("rt_neighbourlist.json")
    do_pbc = pbc == "on"
    # single list, 125 atoms
    atoms = sc_sites(125)
    box = np.diag([5.0] * 3)
    cut = (5.0 / 5) * 1.999
    pairs = orc.nl_classic(0, 125, 0, atoms, box, do_pbc, cut)
    sets = _neigh_sets(pairs, 125)
    exp = g["sets"]["Single list|%s" % pbc]
    for i in range(125):
        assert sorted(sets[i]) == exp[str(i)]
    # two lists / pairs: 124 atoms, A even, B odd
    atoms = sc_sites(124)
    A = np.arange(0, 124, 2)[:62]
    B = np.arange(1, 124, 2)[:62]
    idx = np.concatenate([A, B])
    reordered = atoms[idx]
    for key, mode in (("Two lists", 1), ("List of pairs", 2)):
        pairs = orc.nl_classic(mode, 62, 62, reordered, box, do_pbc, cut)
        sets = _neigh_sets(pairs, 124)
        exp = g["sets"]["%s|%s" % (key, pbc)]
        for slot in range(124):
            got = sorted(int(idx[j]) for j in sets[slot])
            assert got == exp[str(int(idx[slot]))], (key, slot)
    # no NL: every other atom of 27
    pairs = orc.all_pairs(0, 27)
    sets = _neigh_sets(pairs, 27)
    exp = g["sets"]["NoNL|%s" % pbc]
    for i in range(27):
        assert sorted(sets[i]) == exp[str(i)]


def test_cell_nl_equals_classic(orc):
    """The cell-accelerated exact NL returns the classic pair set, sorted."""
    rng = np.random.default_rng(7)
    pos = sc_sites(1728) * 0.31 + rng.normal(0, 0.03, (1728, 3))
    box = np.diag([12 * 0.31] * 3)
    for mode, n0, n1 in ((0, 1728, 0), (1, 864, 864)):
        for do_pbc in (True, False):
            a = orc.nl_classic(mode, n0, n1, pos, box, do_pbc, 0.7)
            b = orc.nl_classic_cells(mode, n0, n1, pos, box, do_pbc, 0.7)
            assert len(a) == len(b)
            a = a[np.lexsort((a[:, 1], a[:, 0]))]
            assert np.array_equal(a, b)


def test_rt_dhenergy(orc, golden):
    """regtest/basic/rt-dhenergy: DHENERGY GROUPA=1-3 GROUPB=4-10 with four
    (I, TEMP, EPSILON) sets, COLVAR and DUMPDERIVATIVES at %6.5f; and
    rt-dhenergy2 (UNITS CHARGE=0.1: charges x10 in plumed units, same values)."""
    import oracle
    g = golden("rt_dhenergy.json")
    na, nb = len(g["group_a"]), len(g["group_b"])
    pairs = orc.all_pairs(oracle.MODE_TWO, na, nb)
    q = np.array(g["charges"])
    assert len(g["frames"]) == len(g["colvar"]) == 5
    for fi, (frame, box) in enumerate(zip(g["frames"], g["box"])):
        B = np.diag(box)
        der = np.array(g["deriv"][fi])
        for ai, lab in enumerate(g["order"]):
            act = g["actions"][lab]
            k, c = orc.dhenergy_constants(act["I"], act["TEMP"], act["EPSILON"])
            p = orc.pairing(oracle.CV_DHENERGY, charges=q, dh=(k, c, act["EPSILON"]))
            s, d, v = orc.cv(p, frame, B, pairs)
            assert abs(s - g["colvar"][fi][ai]) <= 5.01e-6, (fi, lab)
            got = np.concatenate([d.reshape(-1), v.reshape(-1)])
            assert np.abs(got - der[:, ai]).max() <= 5.01e-6, (fi, lab)
            k2, c2 = orc.dhenergy_constants(act["I"], act["TEMP"], act["EPSILON"], unit_charge=0.1)
            p2 = orc.pairing(oracle.CV_DHENERGY, charges=q / 0.1, dh=(k2, c2, act["EPSILON"]))
            s2, _, _ = orc.cv(p2, frame, B, pairs)
            assert abs(s2 - g["colvar_units_charge_0.1"][fi][ai]) <= 5.01e-6, (fi, lab)


def test_rt_ghbfix(orc, golden):
    """regtest/basic/rt-ghbfix: GHBFIX PAIR of atoms 1, 2 at 0.002 i nm apart
    (i = 1..150), TYPES/PARAMS tables read by the product's parser, value
    (colvar c1 = ghbfix + 4.184) and DUMPDERIVATIVES at %8.4f."""
    import oracle
    from plumed2_gb300.siblings import ghbfix_tables
    g = golden("rt_ghbfix.json")
    types, eta = ghbfix_tables(g["types_file"], g["params_file"], energy_units="kcal/mol")
    # the PARAMS rows naming type0/type3 (absent from TYPES) alias id 0
    assert np.allclose(eta, np.array([[5.0, 1.0], [6.0, 0.0]]) * 4.184)
    p = orc.pairing(oracle.CV_GHBFIX, types=types[:2], eta=eta, ghbfix=(0.2, 0.3, 0.8))
    B = np.diag([100.0, 100.0, 100.0])
    for i in range(1, 151):
        z = float("%.6g" % (i * 0.002))  # awk's default output format in the regtest's generator
        s, d, v = orc.cv(p, [[0, 0, 0], [0, 0, z]], B, np.array([[0, 1]], np.uint32))
        assert abs(s + g["c1_minus_ghbfix"] - g["colvar_c1"][i - 1]) <= 5.01e-5, i
        got = np.concatenate([d.reshape(-1), v.reshape(-1)])
        assert np.abs(got - np.array(g["deriv_ghbfix"][i - 1])).max() <= 5.01e-5, i


def test_rt_peratom_coordination(orc, golden):
    """regtest/symfunc/rt-dumpmulti (64 per-atom coordination numbers, %.4f)
    and rt-single-groupb (SPECIESA=1-5 SPECIESB=6 over five frames, %8.4f):
    CONTACT_MATRIX times ones, every pair (no D_MAX)."""
    import oracle
    g = golden("rt_peratom.json")
    d = g["dumpmulti"]
    cn = orc.peratom(d["spec"], d["pos"], np.diag(d["box"]), orc.all_pairs(oracle.MODE_SINGLE, 64))
    assert np.abs(cn - np.array(d["cn"])).max() <= 5.01e-5
    sgb = g["single_groupb"]
    assert len(sgb["frames"]) == 5
    for fi, (fr, bx) in enumerate(zip(sgb["frames"], sgb["box"])):
        cn = orc.peratom(sgb["spec"], fr, np.diag(bx), orc.all_pairs(oracle.MODE_TWO, 5, 1))
        assert np.abs(cn[:5] - np.array(sgb["cn"][fi])).max() <= 5.01e-5, fi


def _cmap_inputs(m, coords):
    cs = m["contacts"]
    pos = np.array([coords(c["atoms"][0]) for c in cs] + [coords(c["atoms"][1]) for c in cs])
    mode = 2 if m["cmdist"] else (1 if m["sum"] else 0)
    return cs, pos, mode


def test_rt_contactmap(orc, golden):
    """regtest/basic/rt28 (CMDIST and components, per-contact switches,
    references and weights; colvar %f, deriv %8.6f) and rt72 (SUM of 278 Q
    contacts in a triclinic box; colvar %f, deriv %12.8f)."""
    g = golden("rt_contactmap.json")
    r = g["rt28"]
    idx = {a: k for k, a in enumerate(r["atoms"])}
    assert len(r["frames"]) == 5
    for fi, (fr, bx) in enumerate(zip(r["frames"], r["box"])):
        B = np.diag(bx)
        res = []
        for m in r["maps"]:
            cs, pos, mode = _cmap_inputs(m, lambda a: fr[idx[a]])
            res.append(orc.contactmap([c["switch"] for c in cs], pos, B, [c["reference"] for c in cs],
                                      [c["weight"] for c in cs], mode))
        (va, da, wa), (vc, _, _) = res
        assert abs(va[0] - r["colvar"][fi][0]) <= 5.01e-7
        assert abs(vc[0] - r["colvar"][fi][1]) <= 5.01e-7 and abs(vc[4] - r["colvar"][fi][2]) <= 5.01e-7
        got = np.concatenate([da.reshape(-1), wa.reshape(-1)])
        assert np.abs(got - np.array(r["deriv_a"][fi])).max() <= 5.01e-7, fi
    r = g["rt72"]
    P = np.array(r["pos"])
    cs, pos, mode = _cmap_inputs(r["map"], lambda a: P[a - 1])
    assert mode == 1 and len(cs) == 278
    v, d, w = orc.contactmap([c["switch"] for c in cs], pos, np.array(r["box"]).reshape(3, 3),
                             [c["reference"] for c in cs], [c["weight"] for c in cs], mode)
    assert abs(v[0] - r["value"]) <= 5.01e-7
    got = np.concatenate([d.reshape(-1), w.reshape(-1)])
    assert np.abs(got - np.array(r["deriv"])).max() <= 5.01e-9


def _box_family(rng, kind):
    """A random box of one of the families of regtest/basic/rt-make-1
    (cubic, orthorhombic, hexagonal, bcc, fcc, generic triclinic with some
    zero entries), rows the lattice vectors."""
    box = np.where(rng.random((3, 3)) > 0.2, 2.0 * rng.random((3, 3)) - 1.0, 0.0)
    if kind in (0, 1):
        box = np.diag(np.diag(box))
        if kind == 0:
            box = np.eye(3) * box[0, 0]
        return box
    if kind == 5:
        return box
    d = 2.0 * rng.random() - 2.0
    rows = {2: [(2.0 * rng.random() - 2.0, 0, 0), (0, d, 0), (0, 0.5 * d, np.sqrt(3.0) * d * 0.5)],
            3: [(d, d, d), (d, -d, d), (d, d, -d)],
            4: [(d, d, 0), (d, 0, d), (0, d, d)]}[kind]
    perm = int(rng.integers(0, 3))
    out = np.zeros((3, 3))
    for k in range(3):
        out[(perm + k) % 3] = rows[k]
    return out


@pytest.mark.parametrize("kind", range(6))
def test_pbc_minimum_image_property(orc, kind):
    """regtest/basic/rt-make-1 restated as a property: for random boxes of
    each family and random vectors (some components zeroed), the image that
    Pbc::distance returns is no longer than any image within two lattice
    shifts of it (the reference's fullSearch check, 1e-15 in squared
    length; failures 0 in logfile.reference)."""
    rng = np.random.default_rng(20 + kind)
    shifts = np.array([(i, j, k) for i in range(-2, 3) for j in range(-2, 3) for k in range(-2, 3)], float)
    nbox = 0
    while nbox < 150:
        box = _box_family(rng, kind)
        if abs(np.linalg.det(box)) < 1e-3:
            continue
        nbox += 1
        v = (rng.random((40, 3)) - 0.5) * 5.0
        v[rng.random((40, 3)) > 0.2] = 0.0
        fast = orc.pbc_distance(box, np.zeros_like(v), v)
        for f in fast:
            full = f + shifts @ box
            assert np.dot(f, f) - (full * full).sum(1).min() <= 1e-15 * max(1.0, np.dot(f, f)), (kind, box, f)


def test_rt_make_celllists(orc, golden):
    """regtest/tools/rt-make-CellLists: link-cell counts of orthorhombic,
    flat and skewed boxes (LinkCells.cpp:99-122), and the cells searched
    from corner, edge, face and middle cells with and without PBC
    (LinkCells::addRequiredCells), sorted as the regtest prints them."""
    g = golden("rt_celllists.json")
    for r in g["counts"]:
        assert orc.linkcells_ncells(np.array(r["box"]).reshape(3, 3), r["cutoff"]) == r["ncells"], r
    for r in g["index_boxes"]:
        assert int(np.prod(orc.linkcells_ncells(np.array(r["box"]).reshape(3, 3), r["cutoff"]))) == r["ncells_total"]
    for r in g["required"]:
        got = orc.linkcells_required(np.array(r["box"]).reshape(3, 3), r["cutoff"], r["cell"], r["pbc"])
        assert got == r["cells"], r


def test_custom_switch_input_the_oracle_cannot_hold_is_refused(orc):
    """A CUSTOM FUNC longer than the oracle's expression buffer, or one missing,
    is an error: a silently shortened expression could still compile into a
    different valid function and pin the checks to the wrong formula."""
    long_func = "FUNC=" + "+".join(["x"] * 80)
    with pytest.raises(ValueError, match="longer"):
        orc.switch("CUSTOM %s R_0=0.3" % long_func)
    with pytest.raises(ValueError, match="without FUNC"):
        orc.switch("CUSTOM R_0=0.3")
    # a short expression still compiles
    orc.switch("CUSTOM FUNC=1/(1+x^6) R_0=0.3")


def metad_numder_case(orc, g):
    """rt-metad-numder replayed: d1 = |min-image(x10 - x1)| per frame (DISTANCE);
    hills deposited after the frames whose step is a multiple of PACE, except
    the first step (MetaD::update, src/bias/MetaD.cpp:2377-2385: no hill on the
    first step), each at the frame's d1 with SIGMA and HEIGHT; frame k feels
    the hills of the frames before it.  Returns d1, the unit vectors and the
    hill centres each frame sees."""
    d, u = [], []
    for fr, bx in zip(g["frames"], g["box"]):
        v = orc.pbc_distance(np.diag(bx), np.array(fr[0]), np.array(fr[1]))[0]
        r = float(np.sqrt(v @ v))
        d.append(r)
        u.append(v / r)
    steps = [k * g["trajectory_stride"] for k in range(len(d))]
    deposit = [k for k, st in enumerate(steps) if st % g["pace"] == 0 and k > 0]
    seen = [[d[j] for j in deposit if j < k] for k in range(len(d))]
    return np.array(d), np.array(u), seen


def test_rt_metad_numder_forces(orc, golden):
    """The hill sum's derivative (oracle.metad_hills, stretched Gaussians as
    METAD's default kernel) times the distance's derivative reproduces the
    reference's analytical forces on atoms 1 and 10 in every frame (%8.4f)."""
    from oracle import metad_hills
    g = golden("rt_metad_numder.json")
    assert g["max_abs_other_forces"] == 0.0
    d, u, seen = metad_numder_case(orc, g)
    for k in range(len(d)):
        n = len(seen[k])
        _, dV = metad_hills([d[k]], [seen[k]], [[g["sigma"]] * n], [[g["height"]] * n], stretch=True)
        f10 = -dV[0] * u[k]  # F = -dV/dd1 * dd1/dx10, dd1/dx10 = u
        assert np.abs(f10 - np.array(g["forces_atom10"][k])).max() <= 5.01e-5, (k, f10, g["forces_atom10"][k])
        assert np.abs(-f10 - np.array(g["forces_atom1"][k])).max() <= 5.01e-5, k
