"""The PLUMED plugin source compiles against PLUMED's own headers (where the
PLUMED source tree is present) and only calls entry points the C ABI declares."""
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PLUGIN = os.path.join(ROOT, "plumed2_gb300", "plugin", "CoordinationGPU.cpp")
sys.path.insert(0, ROOT)
from oracle import REFERENCE_TREE  # noqa: E402

PLUMED_SRC = os.path.join(REFERENCE_TREE, "src")


def test_plugin_uses_declared_abi_only():
    src = open(PLUGIN).read()
    header = open(os.path.join(ROOT, "include", "coordgpu.h")).read()
    used = set(re.findall(r"\b(coord_[a-z0-9_]+)\s*\(", src))
    declared = set(re.findall(r"\b(coord_[a-z0-9_]+)\s*\(", header))
    assert used and used <= declared, used - declared
    assert 'PLUMED_REGISTER_ACTION(CoordinationGPU, "COORDINATION")' in src


@pytest.mark.skipif(not os.path.isdir(os.path.join(PLUMED_SRC, "core")), reason="PLUMED source tree absent")
def test_plugin_compiles_against_plumed_headers():
    p = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I" + PLUMED_SRC, "-I" + os.path.join(ROOT, "include"),
                        PLUGIN], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
