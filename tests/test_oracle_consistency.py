"""Forces against the energy's gradient in the oracle port (CPU).

The reference's PME permanent field adds its Thole correction with the sign
opposite to its energy (MBPolReferenceElectrostaticsForce.cpp:1377-1391
against :2609-2626), so its PME forces are not -dE/dx; with NoCutoff they
are.  The port reproduces the reference by default and takes the consistent
sign under set_pme_fixed_field(True), the mode MBPOL_PME_FIELD_CONSISTENT
selects in the library.  Central differences at h = 1e-4 nm along a random
rigid-M displacement, solver converged to 1e-12 D.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN

oracle = pytest.importorskip("oracle")

M_W = (0.573293118, 0.213353441, 0.213353441)


def _elec(pos, box, alpha, grid):
    L = oracle.port()
    n = pos.shape[0]
    f = np.zeros((n, 3))
    e, it = ctypes.c_double(), ctypes.c_int()
    th = np.array([0.4, 0.4, 0.055, 0.626, 0.055])
    g = np.array(grid, np.int32)
    b = None if box is None else np.ascontiguousarray(box, np.float64)
    rc = L.orc_electrostatics(n, oracle._p(np.ascontiguousarray(pos)), oracle._p(b), 1 if b is not None else 0,
                              alpha, oracle._p(g), 0.9, 1e-12, 500, oracle._p(th), 1, oracle._p(f), ctypes.byref(e),
                              None, ctypes.byref(it), None)
    assert rc == 0
    return e.value, f


def _fd_mismatch(pos, box=None, alpha=0.0, grid=(0, 0, 0), h=1e-4, seed=3):
    """|dE/dh + F.D| / |F.D| for a unit displacement D that moves each M
    site with its O, H1, H2 weights (M is a virtual site)."""
    D = np.random.default_rng(seed).normal(size=pos.shape)
    D[3::4] = M_W[0] * D[0::4] + M_W[1] * D[1::4] + M_W[2] * D[2::4]
    D /= np.linalg.norm(D)
    _, f = _elec(pos, box, alpha, grid)
    fdot = -np.sum(f * D)
    ep = _elec(pos + h * D, box, alpha, grid)[0]
    em = _elec(pos - h * D, box, alpha, grid)[0]
    return abs((ep - em) / (2 * h) - fdot) / abs(fdot)


@pytest.fixture
def pme_water14():
    w = np.load(os.path.join(GOLDEN, "pdb_water14_pme.npz"))
    yield (np.ascontiguousarray(w["positions"]), np.ascontiguousarray(w["box"], np.float64), float(w["alpha"]),
           tuple(int(v) for v in w["grid"]))
    oracle.set_pme_fixed_field(False)


def test_nocutoff_forces_are_energy_gradient():
    c = np.load(os.path.join(GOLDEN, "elec_cluster14_seed0.npz"))
    assert _fd_mismatch(np.ascontiguousarray(c["positions"])) < 1e-6


def test_pme_reference_sign_forces_are_not_energy_gradient(pme_water14):
    pos, box, alpha, grid = pme_water14
    oracle.set_pme_fixed_field(False)
    assert _fd_mismatch(pos, box, alpha, grid) > 1e-3


def test_pme_consistent_sign_forces_are_energy_gradient(pme_water14):
    pos, box, alpha, grid = pme_water14
    oracle.set_pme_fixed_field(True)
    assert _fd_mismatch(pos, box, alpha, grid) < 1e-6
