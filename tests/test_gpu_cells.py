"""GPU: the O-O lists built from cells against the oracle port's all-pairs
lists, on a periodic box large enough for a cell grid.

1000 waters on a jittered 10^3 lattice in a 3.104 nm box: the two-body
list (0.65 nm) bins into 4 cells per dimension, the three-body list
(0.45 nm) into 6, dispersion and the shared list (0.9 nm) into 3.
Counts must be equal, energies within 2e-6 relative, forces within 1e-4
relative RMS (the tolerances of the per-term parity tests); the complete
trimer rule's count is checked against a count from the O-O distance
matrix (triples with at least two of three distances <= 0.45 nm:
sum over waters of C(degree, 2) minus twice the triangles).
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_rms
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import systems

pytestmark = pytest.mark.gpu
oracle = pytest.importorskip("oracle")


@pytest.fixture(scope="module")
def box1000():
    return systems.lattice_box(10, 10, 10, 31.04, 1000, seed=3)


def _gpu(ws, terms, trimer_rule=0):
    s = mb.create_mbpol_system(ws, terms=terms, trimer_rule=trimer_rule)
    ctx = mb.Context(s)
    ctx.setPositions(ws.positions)
    st = ctx.getState()
    return st, ctx.getCounts()


_PORT = {}


def _port(ws, term):
    if term in _PORT:
        return _PORT[term]
    L = oracle.port()
    pos = np.ascontiguousarray(ws.positions, np.float64)
    nw = ws.num_waters
    w = np.ascontiguousarray(np.stack([4 * np.arange(nw), 4 * np.arange(nw) + 1, 4 * np.arange(nw) + 2], 1), np.int32)
    box = np.ascontiguousarray(ws.box, np.float64)
    f = np.zeros_like(pos)
    p = oracle._p
    if term == "twobody":
        n = ctypes.c_long()
        e = L.orc_twobody(nw, p(w), p(pos), p(box), 0.65, p(f), ctypes.byref(n))
    elif term == "threebody":
        n, ns = ctypes.c_long(), ctypes.c_long()
        e = L.orc_threebody(nw, p(w), p(pos), p(box), 0.45, 1, p(f), ctypes.byref(n), ctypes.byref(ns))
    else:
        n = ctypes.c_long(0)
        e = L.orc_dispersion(nw, p(w), p(pos), p(box), 0.9, p(f))
    _PORT[term] = (e, f, n.value)
    return _PORT[term]


@pytest.mark.parametrize("term,slot,count", [("twobody", 1, 0), ("threebody", 2, 1), ("dispersion", 4, None)])
def test_cell_lists_vs_all_pairs_oracle(box1000, term, slot, count):
    st, counts = _gpu(box1000, (term,))
    e_ref, f_ref, n_ref = _port(box1000, term)
    e = st.term_energies[slot]
    print(term, "E %.8f oracle %.8f rel %.2e | F relrms %.2e | count %s oracle %d" % (
        e, e_ref, abs(e - e_ref) / abs(e_ref), rel_rms(st.getForces(), f_ref),
        counts[count] if count is not None else "-", n_ref))
    assert abs(e - e_ref) <= 2e-6 * abs(e_ref)
    assert rel_rms(st.getForces(), f_ref) <= 1e-4
    if count is not None:
        assert counts[count] == n_ref


def test_shared_cell_lists_match_separate_terms(box1000):
    """2B + 3B + dispersion in one evaluation take the shared list pass."""
    st, counts = _gpu(box1000, ("twobody", "threebody", "dispersion"))
    for term, slot in (("twobody", 1), ("threebody", 2), ("dispersion", 4)):
        e_ref = _port(box1000, term)[0]
        assert abs(st.term_energies[slot] - e_ref) <= 2e-6 * abs(e_ref), term


def test_complete_trimer_count(box1000):
    _, counts = _gpu(box1000, ("threebody",), trimer_rule=1)
    o = box1000.positions[0::4]
    L = np.asarray(box1000.box, float)
    d = o[:, None, :] - o[None, :, :]
    d -= L * np.round(d / L)
    A = ((d * d).sum(-1) <= 0.45 ** 2).astype(np.int64)
    np.fill_diagonal(A, 0)
    deg = A.sum(1)
    triangles = np.trace(A @ A @ A) // 6
    expect = int((deg * (deg - 1) // 2).sum() - 2 * triangles)
    print("complete-rule trimers", counts[1], "expected", expect)
    assert counts[1] == expect
