"""The PLUMED plugin's own C++ code (plumed2_gb300/plugin/CoordinationGPU.cpp)
compiled unchanged against the harness's minimal action interface
(tests/plugin_host): the keyword checks that run before any device work, on
CPU.  The numerics through the plugin are in test_gpu_plugin_host.py."""
import numpy as np
import pytest

from tests.plugin_host import harness

BOX = np.eye(3) * 3.0


def _err(line):
    pos = np.zeros((1, 10, 3))
    with pytest.raises(harness.PluginError) as e:
        harness.run(line, pos, BOX[None])
    return str(e.value)


def test_harness_builds_and_registers_the_plugin_directives():
    harness.load()
    assert "unknown directive" in _err("c: NOT_AN_ACTION GROUPA=1-10")


def test_plugin_keyword_errors_as_the_reference():
    # CoordinationBase.cpp:71 (one NL version at a time)
    assert "Please activate only one of the two version of the NL" in _err(
        "c: COORDINATION GROUPA=1-10 R_0=0.3 NLIST NLISTCELLS NL_CUTOFF=1 NL_STRIDE=1")
    # Coordination.cpp:145-147 (R_0 > 0), raised by coord_create through the plugin's error()
    assert "R_0 should be explicitly specified and positive" in _err("c: COORDINATION GROUPA=1-10")
    # Action::checkRead: words nobody parsed
    assert "cannot understand the following words" in _err("c: COORDINATION GROUPA=1-10 R_0=0.3 FOO=1")
    # the error names the action and its label
    msg = _err("mylabel: COORDINATION GROUPA=1-10")
    assert "COORDINATION" in msg and "mylabel" in msg
