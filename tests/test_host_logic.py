"""Host-side logic of the §8f actions, on the CPU: keyword reading and the
reference's error messages (raised before any device call), the GHBFIX
tables, the energy units, and the bench's pair accounting."""
import numpy as np
import pytest

from plumed2_gb300.siblings import energy_unit, ghbfix_tables, table_rows


def test_energy_units():
    """Units::setEnergy (tools/Units.cpp:40-60)."""
    assert energy_unit("kj/mol") == 1.0
    assert energy_unit("kcal/mol") == 4.184
    assert energy_unit("j/mol") == 0.001
    assert energy_unit("eV") == 96.48530749925792
    assert energy_unit("Ha") == 2625.499638
    assert energy_unit("2.5") == 2.5
    with pytest.raises(ValueError, match="case sensitive"):
        energy_unit("KCAL/MOL")
    with pytest.raises(ValueError, match="positive"):
        energy_unit("-1")


def test_table_rows():
    text = "#! FIELDS itype jtype eta\n# a comment\n\nA B 1.5\n#! SET x 1\nB A 2.0\n"
    assert table_rows(text, ["itype", "eta"]) == [{"itype": "A", "eta": "1.5"}, {"itype": "B", "eta": "2.0"}]
    with pytest.raises(ValueError, match="FIELDS"):
        table_rows("A B 1\n", ["itype"])
    with pytest.raises(ValueError, match="no field"):
        table_rows("#! FIELDS itype\nA\n", ["eta"])


def test_ghbfix_tables_ids_and_aliasing():
    """Type ids in order of first appearance; a PARAMS name that TYPES never
    named takes id 0 (std::map::operator[] in GHBFIX.cpp:164); ENERGY_UNITS
    scales eta to the plumed unit."""
    types = "#! FIELDS itype\nO\nH\nH\nN\nO\n"
    params = "#! FIELDS itype jtype eta\nO H 1.0\nH O 2.0\nN N 3.0\nX H 4.0\n"
    t, eta = ghbfix_tables(types, params)
    assert list(t) == [0, 1, 1, 2, 0]
    want = np.zeros((3, 3))
    want[0, 1] = 4.0  # X aliases O (id 0) and is read last
    want[1, 0] = 2.0
    want[2, 2] = 3.0
    assert np.array_equal(eta, want)
    t2, eta2 = ghbfix_tables(types, params, energy_units="kcal/mol", plumed_energy=2.0)
    assert np.array_equal(t2, t) and np.allclose(eta2, want * 4.184 / 2.0)
    with pytest.raises(ValueError, match="empty TYPES"):
        ghbfix_tables("#! FIELDS itype\n", params)


def test_contactmap_keyword_errors():
    """ContactMap::ContactMap's reading order and messages (ContactMap.cpp:147-287)."""
    from plumed2_gb300.action import ContactMap
    with pytest.raises(ValueError, match="You cannot use SUM and CMDIST together"):
        ContactMap("ATOMS1=1,2 SWITCH={RATIONAL R_0=1} SUM CMDIST")
    with pytest.raises(ValueError, match="ATOMS2 keyword has the wrong number of atoms"):
        ContactMap("ATOMS1=1,2 ATOMS2=3 SWITCH={RATIONAL R_0=1}")
    with pytest.raises(ValueError, match="missing SWITCH2 keyword"):
        ContactMap("ATOMS1=1,2 ATOMS2=3,4 ATOMS3=5,6 SWITCH1={RATIONAL R_0=1}")
    with pytest.raises(ValueError, match="no switching function specified use SWITCH keyword"):
        ContactMap("ATOMS1=1,2")
    with pytest.raises(ValueError, match="with CMDIST one must use REFERENCE"):
        ContactMap("ATOMS1=1,2 SWITCH={RATIONAL R_0=1} CMDIST")
    with pytest.raises(ValueError, match="cannot read flag"):
        ContactMap("ATOMS1=1,2 SWITCH={RATIONAL R_0=1} MEAN")
    with pytest.raises(ValueError, match="cannot read keyword"):
        ContactMap("ATOMS1=1,2 SWITCH={RATIONAL R_0=1} FOO=3")


def test_coordinationnumber_keyword_errors():
    """CoordinationNumbers::CoordinationNumbers (CoordinationNumbers.cpp:327-349, 284-296)."""
    from plumed2_gb300.action import CoordinationNumbers
    with pytest.raises(ValueError, match="missing atoms input use SPECIES or SPECIESA/SPECIESB"):
        CoordinationNumbers("SWITCH={RATIONAL R_0=1}")
    with pytest.raises(ValueError, match="missing atoms input"):
        CoordinationNumbers("SPECIESA=1-4 SWITCH={RATIONAL R_0=1}")
    with pytest.raises(ValueError, match="missing switching function parameters use SWITCH/R_0"):
        CoordinationNumbers("SPECIES=1-10")
    with pytest.raises(ValueError, match="cannot read keyword"):
        CoordinationNumbers("SPECIES=1-10 R_0=1 NLIST=1")


def test_sibling_keyword_surface():
    """DHENERGY and GHBFIX take CoordinationBase's keywords plus their own,
    not COORDINATION's switching-function keywords."""
    from plumed2_gb300.action import GHBFIX, DHEnergy
    with pytest.raises(ValueError, match="cannot read keyword SWITCH"):
        DHEnergy("GROUPA=1-4 SWITCH={RATIONAL R_0=1}")
    with pytest.raises(ValueError, match="cannot read keyword R_0"):
        DHEnergy("GROUPA=1-4 R_0=1")
    with pytest.raises(ValueError, match="keyword C is compulsory"):
        GHBFIX("GROUPA=1-4 D_0=0.2 D_MAX=0.3", types_text="#! FIELDS itype\nA\n", params_text="")


def test_e2e_pair_accounting():
    import bench
    # lists built at step 0 serve steps 1..9; the step-10 rebuild serves 10..
    assert bench.e2e_pairs(100, 110, 5) == 500
    assert bench.e2e_pairs(100, 110, 10) == 9 * 100 + 110
    assert bench.e2e_pairs(100, 110, 12) == 9 * 100 + 3 * 110


def test_atom_ranges():
    """Tools::interpretRanges (tools/Tools.cpp:559-601): a-b:stride runs from a
    to b inclusive, downwards with a negative stride; a stride of the wrong
    sign is an error, with the reference's message."""
    from plumed2_gb300.action import parse_atom_list
    assert parse_atom_list("1-10:3") == [0, 3, 6, 9]
    assert parse_atom_list("108-1:-1") == list(range(107, -1, -1))
    assert parse_atom_list("108-50:-1,1-49") == list(range(107, 48, -1)) + list(range(49))
    assert parse_atom_list("5-5,3") == [4, 2]
    for bad in ("10-1", "1-10:-1", "1-10:0", "10-1:2"):
        with pytest.raises(ValueError, match="interpreting ranges %s, stride should be positive" % bad):
            parse_atom_list(bad)
