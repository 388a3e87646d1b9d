"""CPU: the C-ABI library exists (after build()), loads, and exports every
function declared in include/mbpol_gb300.h.  No compute call is made."""
import ctypes
import os
import re

import pytest

from conftest import ROOT
from mbpol_openmm_plugin_gb300 import _capi


def declared_functions():
    src = open(os.path.join(ROOT, "include", "mbpol_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mbpol_[a-z0-9_]+)\s*\(", src)) - {"mbpol_status"})


def test_header_matches_binding_list():
    assert set(declared_functions()) == set(_capi.EXPORTED)


def test_library_exports_all_symbols():
    if not os.path.exists(_capi.LIB_PATH):
        pytest.skip("library not built")
    lib = ctypes.CDLL(_capi.LIB_PATH)
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_status_strings_without_gpu():
    if not os.path.exists(_capi.LIB_PATH):
        pytest.skip("library not built")
    lib = _capi.load()
    assert lib.mbpol_status_string(3) == b"induced dipoles did not converge"


def test_cxx_layer_compiles_and_links(tmp_path):
    """The C++ Force-class header compiles against the C ABI and links."""
    import shutil
    import subprocess
    if not os.path.exists(_capi.LIB_PATH) or shutil.which("g++") is None:
        pytest.skip("library not built or no g++")
    exe = tmp_path / "example_water2"
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cxx", "example_water2.cpp"), "-o", str(exe),
                           "-L", os.path.dirname(_capi.LIB_PATH), "-lmbpol_gb300",
                           "-Wl,-rpath," + os.path.dirname(_capi.LIB_PATH)])
    assert exe.exists()


def test_noalloc_capacity_and_argument_checks_without_gpu():
    """The no-allocation two-body entry point: the capacity in the header
    matches the binding, and oversize or negative dimer counts are rejected
    on the host before any CUDA call."""
    src = open(os.path.join(ROOT, "include", "mbpol_gb300.h")).read()
    m = re.search(r"#define\s+MBPOL_NOALLOC_MAX_DIMERS\s+(\d+)", src)
    assert m and int(m.group(1)) == _capi.NOALLOC_MAX_DIMERS
    if not os.path.exists(_capi.LIB_PATH):
        pytest.skip("library not built")
    lib = _capi.load()
    fn = lib.mbpol_twobody_dimers_noalloc
    assert fn(None, None, None, _capi.NOALLOC_MAX_DIMERS + 1, None, None, None, None) == 5  # MBPOL_ERR_CAPACITY
    assert fn(None, None, None, -1, None, None, None, None) == 1  # MBPOL_ERR_INVALID_ARGUMENT
    assert fn(None, None, None, 0, None, None, None, None) == 0
