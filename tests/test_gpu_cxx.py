"""GPU: the C++ Force-class layer end to end (two waters,
TestReferenceMBPolTwoBodyForce.cpp:99-127, E = 6.14207815 kcal/mol)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT
from mbpol_openmm_plugin_gb300 import _capi

pytestmark = pytest.mark.gpu


def test_cxx_two_water_known_answer(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = tmp_path / "example_water2"
    libdir = os.path.dirname(_capi.LIB_PATH)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cxx", "example_water2.cpp"), "-o", str(exe),
                           "-L", libdir, "-lmbpol_gb300", "-Wl,-rpath," + libdir])
    out = subprocess.check_output([str(exe)], text=True).strip()
    assert abs(float(out) - 6.14207815) < 1e-3, out
