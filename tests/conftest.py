import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


GOLDEN = os.path.join(ROOT, "tests", "golden")


def rel_rms(f, ref):
    import numpy as np
    return float(np.sqrt(((f - ref) ** 2).sum()) / max(np.sqrt((ref ** 2).sum()), 1e-300))
