"""The C ABI without a GPU: the library loads, exports every declared symbol,
validates keywords with the reference's messages, and sets up switching
functions bit-identically to the reference (via the oracle, itself pinned to
the reference)."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "coordgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(coord_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from plumed2_gb300 import _lib
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    from plumed2_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(coord_[a-z0-9_]+)", out))
    declared = _declared()
    assert len(declared) >= 25
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    for s in declared:
        getattr(lib, s)  # resolvable through ctypes


def test_host_path_without_a_call(lib):
    # no context, or no host-array call yet: -1; the codes the header defines
    assert lib.coord_host_path(None) == -1
    from plumed2_gb300.action import Coordination
    assert Coordination.HOST_PATHS == {-1: None, 0: "staged", 1: "direct", 2: "chunked"}
    hdr = open(os.path.join(ROOT, "include", "coordgpu.h")).read()
    for name, code in (("STAGED", 0), ("DIRECT", 1), ("CHUNKED", 2)):
        assert re.search(r"#define COORD_HOST_PATH_%s %d\b" % (name, code), hdr)


def test_status_strings(lib):
    assert lib.coord_status_string(0) == b"ok"
    assert lib.coord_status_string(2) == b"CUDA error"


@pytest.mark.parametrize("line,msg", [
    ("GROUPA=1-10 NLIST R_0=1", "NL_CUTOFF should be explicitly specified and positive"),
    ("GROUPA=1-10 NLIST NL_CUTOFF=1 R_0=1", "NL_STRIDE should be explicitly specified and positive"),
    ("GROUPA=1-10 NLIST NL_CUTOFF=-1 NL_STRIDE=1 R_0=1", "NL_CUTOFF should be explicitly specified and positive"),
    ("GROUPA=1-10 R_0=0", "R_0 should be explicitly specified and positive"),
    ("GROUPA=1-10", "R_0 should be explicitly specified and positive"),
    ("GROUPA=1-10 SWITCH={RATIONAL R_0=1 FOO=2}", "rogue keywords"),
    ("GROUPA=1-10 SWITCH={NOTASWITCH R_0=1}", "cannot understand switching function type"),
    ("GROUPA=1-10 SWITCH={RATIONAL D_0=1}", "R_0 is required for RATIONAL"),
    ("GROUPA=1 GROUPB=2 PAIR NLISTCELLS NL_CUTOFF=1 NL_STRIDE=1 R_0=1",
     "Pair is not compatible with the CELLS implementation"),
    ("GROUPA=1 NLIST NLISTCELLS NL_CUTOFF=1 NL_STRIDE=1 R_0=1", "only one of the two version of the NL"),
])
def test_keyword_errors(line, msg):
    from plumed2_gb300.action import Coordination
    with pytest.raises(ValueError, match=re.escape(msg)):
        Coordination(line)


def test_custom_switch_errors():
    """CUSTOM (lepton) expressions the reference refuses are refused with its
    messages (leptonSwitch::funcAndDeriv, SwitchingFunction.cpp:566-585);
    lepton's parse errors are reported as such."""
    from plumed2_gb300.action import Coordination
    Coordination("GROUPA=1-10 SWITCH={CUSTOM FUNC=1/(1+x^6) R_0=1}").close()
    Coordination("GROUPA=1-10 SWITCH={CUSTOM FUNC={1 / (1 + x2^3)} R_0=1}").close()
    for func, msg in (("x*x2", "only ONE argument"), ("y+x", "only ONE argument"), ("foo(x)", "unknown function"),
                      ("(1+x", "unbalanced"), ("1/(1+x^6))", "unexpected")):
        with pytest.raises(ValueError, match=re.escape(msg)):
            Coordination("GROUPA=1-10 SWITCH={CUSTOM FUNC=%s R_0=1}" % func)


def test_atom_list_parsing():
    from plumed2_gb300.action import parse_atom_list, split_line
    assert parse_atom_list("1-5") == [0, 1, 2, 3, 4]
    assert parse_atom_list("1,3,5-9:2") == [0, 2, 4, 6, 8]
    assert split_line("c: COORDINATION GROUPA=1-3 SWITCH={RATIONAL R_0=1 D_MAX=2}") == [
        "c:", "COORDINATION", "GROUPA=1-3", "SWITCH={RATIONAL R_0=1 D_MAX=2}"]


SPECS = [
    ("SWITCH={RATIONAL R_0=0.30 D_0=0.0 NN=6 MM=12 D_MAX=1.0}", "RATIONAL R_0=0.30 D_0=0.0 NN=6 MM=12 D_MAX=1.0"),
    ("SWITCH={RATIONAL R_0=1.3 NN=6 MM=10 D_MAX=2.6}", "RATIONAL R_0=1.3 NN=6 MM=10 D_MAX=2.6"),
    ("SWITCH={RATIONAL R_0=1.3 NN=5 MM=11 D_MAX=2.6}", "RATIONAL R_0=1.3 NN=5 MM=11 D_MAX=2.6"),
    ("SWITCH={RATIONAL R_0=1.3 NN=5 D_MAX=2.6}", "RATIONAL R_0=1.3 NN=5 D_MAX=2.6"),
    ("SWITCH={RATIONAL R_0=0.3 NN=6 MM=12}", "RATIONAL R_0=0.3 NN=6 MM=12"),
    ("SWITCH={RATIONAL R_0=1.3 NN=6 MM=10 D_MAX=2.6 NOSTRETCH}", "RATIONAL R_0=1.3 NN=6 MM=10 D_MAX=2.6 NOSTRETCH"),
    ("SWITCH={EXP R_0=0.8 D_0=0.5 D_MAX=2.6}", "EXP R_0=0.8 D_0=0.5 D_MAX=2.6"),
    ("SWITCH={GAUSSIAN R_0=1.0 D_0=0.0 D_MAX=2.6}", "GAUSSIAN R_0=1.0 D_0=0.0 D_MAX=2.6"),
    ("SWITCH={GAUSSIAN R_0=1.0 D_0=0.3 D_MAX=2.6}", "GAUSSIAN R_0=1.0 D_0=0.3 D_MAX=2.6"),
    ("SWITCH={Q R_0=1.0 D_0=0.3 BETA=5.0 LAMBDA=1.0 REF=1.3 D_MAX=2.6}",
     "Q R_0=1.0 D_0=0.3 BETA=5.0 LAMBDA=1.0 REF=1.3 D_MAX=2.6"),
    ("SWITCH={TANH R_0=1.3 D_MAX=2.6}", "TANH R_0=1.3 D_MAX=2.6"),
    ("SWITCH={SMAP R_0=1.3 A=3 B=2 D_MAX=2.6}", "SMAP R_0=1.3 A=3 B=2 D_MAX=2.6"),
    ("SWITCH={CUBIC D_MAX=2.6 D_0=0.6}", "CUBIC D_MAX=2.6 D_0=0.6"),
    ("SWITCH={COSINUS R_0=2.6}", "COSINUS R_0=2.6"),
    ("R_0=0.3", "R0SYNTAX 6 0 0.3 0.0"),
    ("R_0=1.0 NN=7 D_0=0.1", "R0SYNTAX 7 0 1.0 0.1"),
    ("R_0=0.4 NN=8 MM=14 D_0=0.05", "R0SYNTAX 8 14 0.4 0.05"),
]


@pytest.mark.parametrize("kw,spec", SPECS)
def test_host_switch_setup_matches_reference(orc, kw, spec):
    """Stretch/shift and every (sigma, dfunc) from the library's host set-up
    equal the oracle's (== the reference's) bit for bit."""
    from plumed2_gb300.action import Coordination
    c = Coordination("GROUPA=1-2 " + kw)
    x = np.linspace(0.0, 3.0, 2001)
    for squared in (True, False):
        xx = x * x if squared else x
        f1, d1 = c.switch(xx, squared)
        f2, d2 = orc.switch_eval(spec, xx, squared)
        if "EXP" in spec or "GAUSSIAN" in spec or "Q " in spec or "TANH" in spec or "SMAP" in spec \
                or "COSINUS" in spec:
            # libm transcendental functions: host glibc on both sides, same bits
            assert np.array_equal(f1, f2) and np.array_equal(d1, d2)
        else:
            assert np.array_equal(f1, f2) and np.array_equal(d1, d2)
