"""CPU: the trie split of the polynomial walks (csrc/poly_df.cu, make_split)
covers the trie exactly once for two and three parts per unit and for
uneven cuts.  The harness is compiled on the host with nvcc; no GPU is
used."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "mbpol_openmm_plugin_gb300", "csrc")
BUILD = os.path.join(ROOT, "mbpol_openmm_plugin_gb300", "_build")

CASES = [
    ("three_default", []),
    ("two_parts", ["-DMBPOL_WALK_PARTS=2", "-DMBPOL_WALK_CUTS_2B={0.57}", "-DMBPOL_WALK_CUTS_3B={0.54}"]),
    ("three_late_cuts", ["-include", os.path.join(HERE, "cxx", "walk_cuts_late.h")]),
]


@pytest.mark.parametrize("name,flags", CASES)
def test_walk_split_covers_trie(name, flags, tmp_path):
    nvcc = shutil.which(os.environ.get("NVCC", "nvcc"))
    if nvcc is None:
        pytest.skip("nvcc not found")
    if not os.path.exists(os.path.join(CSRC, "gen", "poly3b_tables.inc")):
        pytest.skip("generated trie tables missing (run the build first)")
    exe = str(tmp_path / name)
    subprocess.run([nvcc, "-std=c++17", "-O1", "-I", CSRC, "-I", BUILD] + flags +
                   [os.path.join(HERE, "cxx", "walk_split_check.cu"), "-o", exe],
                   check=True, capture_output=True, timeout=600)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
