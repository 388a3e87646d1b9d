"""GPU parity: one-, two-, three-body and dispersion through the C ABI vs
the FP64 reference (fixtures from the compiled Reference platform and the
reference's own known answers).

Tolerances (FP32 bulk arithmetic, FP64 accumulation):
  forces   relative RMS error <= 1e-4 per term
  energy   relative error <= 1e-6 (one-body, FP64), <= 2e-6 (two-body,
           dispersion and the three-body double-float walk: FP32 polynomial /
           pair arithmetic, FP64 sums); three-body on the tensor cores
           <= 2e-5 relative + 5e-5 kJ/mol (fp16 operand pieces with FP32
           sums: ~1e-6 kcal/mol per trimer, largely random; the total
           energy, 10-100x the three-body term, stays within 1e-7 -- the
           full-model tests hold it to the metric's 1e-6)
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import systems

pytestmark = pytest.mark.gpu
KCAL = 4.184
FORCE_TOL = 1e-4
E_TOL = {"e1": 1e-6, "e2": 2e-6, "e3": 2e-6, "edisp": 2e-6}


E3_TC_TOL, E3_TC_ABS = 2e-5, 5e-5


def run(ws_pos, box, terms, trimer_rule=0, cut2=0.65, cut3=0.45, evaluator=mb.MBPolThreeBodyForce.TensorCores):
    ws = systems.WaterSystem(ws_pos, box, 0, "fixture")
    s = mb.create_mbpol_system(ws, terms=terms, trimer_rule=trimer_rule)
    for f in s.forces:
        if isinstance(f, mb.MBPolTwoBodyForce):
            f.setCutoff(cut2)
        if isinstance(f, mb.MBPolThreeBodyForce):
            f.setCutoff(cut3)
            f.setPolynomialEvaluator(evaluator)
    ctx = mb.Context(s)
    ctx.setPositions(ws_pos)
    st = ctx.getState()
    return st, ctx


TERMS = {"e1": ("onebody", 0), "e2": ("twobody", 1), "e3": ("threebody", 2), "edisp": ("dispersion", 4)}
FKEY = {"e1": "f1", "e2": "f2", "e3": "f3", "edisp": "fdisp"}


@pytest.mark.parametrize("name", ["cluster14_seed0", "cluster14_seed1", "box256_seed0", "cluster64_seed2"])
@pytest.mark.parametrize("term", ["e1", "e2", "e3", "edisp"])
def test_term_vs_reference(name, term):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    box = d["box"] if bool(d["periodic"]) else None
    tname, slot = TERMS[term]
    st, ctx = run(d["positions"], box, (tname,))
    e = st.term_energies[slot]
    eref = float(d[term])
    f = st.getForces()
    fref = d[FKEY[term]]
    print(name, term, "E", e, eref, "rel", abs(e - eref) / abs(eref), "F relrms", rel_rms(f, fref))
    if term == "e3":
        assert abs(e - eref) <= E3_TC_TOL * abs(eref) + E3_TC_ABS
    else:
        assert abs(e - eref) <= E_TOL[term] * abs(eref)
    assert rel_rms(f, fref) <= FORCE_TOL
    if term == "e2":
        assert ctx.getCounts()[0] == int(d["npairs"])
    if term == "e3":
        assert ctx.getCounts()[1] == int(d["ntrip"])


@pytest.mark.parametrize("name", ["cluster14_seed0", "cluster14_seed1", "box256_seed0", "cluster64_seed2"])
def test_threebody_walk_vs_reference(name):
    """The double-float walk (MBPOL_POLY3B_WALK) at the walk's tolerance."""
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    box = d["box"] if bool(d["periodic"]) else None
    st, ctx = run(d["positions"], box, ("threebody",), evaluator=mb.MBPolThreeBodyForce.DoubleFloatWalk)
    e, eref = st.term_energies[2], float(d["e3"])
    print(name, "walk E3", e, eref, "rel", abs(e - eref) / abs(eref), "F relrms", rel_rms(st.getForces(), d["f3"]))
    assert abs(e - eref) <= 2e-6 * abs(eref)
    assert rel_rms(st.getForces(), d["f3"]) <= FORCE_TOL


@pytest.mark.parametrize("tensor", ["tcgen05", "mma.sync"])
@pytest.mark.parametrize("name", ["box256_seed0", "pdb_water256_pme", "box4096_seed0"])
def test_threebody_tensor_vs_walk(name, tensor):
    """The tensor-core evaluations (tcgen05, and the legacy mma.sync path)
    against the double-float walk on the same trimers: energy and forces of
    the three-body term."""
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    box = d["box"] if bool(d["periodic"]) else None
    T = mb.MBPolThreeBodyForce
    res = []
    for ev in (T.TensorCores if tensor == "tcgen05" else T.TensorCoresMmaSync, T.DoubleFloatWalk):
        st, ctx = run(d["positions"], box, ("threebody",), evaluator=ev)
        res.append((st.term_energies[2], st.getForces()))
    (e_tc, f_tc), (e_w, f_w) = res
    print(name, tensor, "E3", e_tc, "walk", e_w, "rel", abs(e_tc - e_w) / abs(e_w), "F relrms", rel_rms(f_tc, f_w))
    assert abs(e_tc - e_w) <= E3_TC_TOL * abs(e_w) + E3_TC_ABS
    assert rel_rms(f_tc, f_w) <= 2e-5


def test_threebody_tcgen05_repeatable_and_ragged():
    """The tcgen05 kernel on a trimer count that leaves a ragged last tile
    and more tiles than blocks (box4096 fixture): repeated evaluations and a
    second context agree to the FP64 atomics' summation order (the kernel's
    own per-trimer sums have a fixed order)."""
    d = np.load(os.path.join(GOLDEN, "box4096_seed0.npz"))
    T = mb.MBPolThreeBodyForce
    st1, ctx = run(d["positions"], d["box"], ("threebody",), evaluator=T.TensorCores)
    assert ctx.getCounts()[1] % 128 != 0
    ctx.setPositions(d["positions"])
    st2 = ctx.getState()
    st3, _ = run(d["positions"], d["box"], ("threebody",), evaluator=T.TensorCores)
    e1 = st1.term_energies[2]
    for st in (st2, st3):
        assert abs(st.term_energies[2] - e1) <= 1e-12 * abs(e1)
        assert rel_rms(st.getForces(), st1.getForces()) <= 1e-12


def _known(key):
    known = json.load(open(os.path.join(GOLDEN, "reference_known_answers.json")))[key]
    pos = np.array(known["positions_A"]) * 0.1
    return pos, known


@pytest.mark.parametrize("box_nm,offset", [(0.0, False), (50.0, False), (50.0, True)])
def test_twobody_known_answer(box_nm, offset):
    """TestReferenceMBPolTwoBodyForce.cpp:59-172: cluster, PBC 50 nm, offset by one box."""
    pos, known = _known("twobody_water2")
    if offset:
        pos[3:6, 1] += box_nm
    s = mb.System()
    for _ in range(6):
        s.addParticle(1.0)
    f = mb.MBPolTwoBodyForce()
    f.setCutoff(10.0 if box_nm == 0 else 10.0)
    f.addParticle([0, 1, 2])
    f.addParticle([3, 4, 5])
    if box_nm > 0:
        s.setDefaultPeriodicBoxVectors((box_nm, 0, 0), (0, box_nm, 0), (0, 0, box_nm))
        f.setNonbondedMethod(mb.MBPolTwoBodyForce.CutoffPeriodic)
    else:
        f.setNonbondedMethod(mb.MBPolTwoBodyForce.CutoffNonPeriodic)
    s.addForce(f)
    ctx = mb.Context(s)
    ctx.setPositions(pos)
    st = ctx.getState()
    assert abs(st.getPotentialEnergy() / KCAL - known["expected_energy_kcal"]) < 1e-3
    g = -st.getForces() / (KCAL * 10)
    assert np.allclose(g, np.array(known["expected_gradient_kcal_A"]), atol=1e-3)


@pytest.mark.parametrize("box_nm,offset", [(0.0, False), (50.0, False), (50.0, True)])
def test_threebody_known_answer(box_nm, offset):
    """TestReferenceMBPolThreeBodyForce.cpp:57-211."""
    pos, known = _known("threebody_water3")
    if offset:
        pos[3:6, 1] += box_nm
    s = mb.System()
    for _ in range(9):
        s.addParticle(1.0)
    f = mb.MBPolThreeBodyForce()
    f.setCutoff(10.0)
    for w in range(3):
        f.addParticle([3 * w, 3 * w + 1, 3 * w + 2])
    if box_nm > 0:
        s.setDefaultPeriodicBoxVectors((box_nm, 0, 0), (0, box_nm, 0), (0, 0, box_nm))
        f.setNonbondedMethod(mb.MBPolThreeBodyForce.CutoffPeriodic)
    else:
        f.setNonbondedMethod(mb.MBPolThreeBodyForce.CutoffNonPeriodic)
    s.addForce(f)
    ctx = mb.Context(s)
    ctx.setPositions(pos)
    st = ctx.getState()
    assert abs(st.getPotentialEnergy() / KCAL - known["expected_energy_kcal"]) < 1e-3
    g = -st.getForces() / (KCAL * 10)
    assert np.allclose(g, np.array(known["expected_gradient_kcal_A"]), atol=1e-3)


def test_onebody_known_answer():
    """TestReferenceMBPolOneBodyForce.cpp:53-143."""
    pos, known = _known("onebody_water1")
    s = mb.System()
    for _ in range(3):
        s.addParticle(1.0)
    f = mb.MBPolOneBodyForce()
    f.addOneBody([0, 1, 2])
    s.addForce(f)
    ctx = mb.Context(s)
    ctx.setPositions(pos)
    st = ctx.getState()
    assert abs(st.getPotentialEnergy() / KCAL - known["expected_energy_kcal"]) < 1e-4
    g = -st.getForces() / (KCAL * 10)
    assert np.allclose(g, np.array(known["expected_gradient_kcal_A"]), atol=1e-4)


def test_trimer_chain_rule():
    """TestReferenceThreeNeighborList.cpp:42-78: an open trimer counts only
    when its shared vertex has the middle index (chain rule); the complete
    rule counts it either way."""
    # three waters on a line-ish open chain, O-O 0.3 nm, vertex = middle or last
    base = systems.cluster(3, seed=5, radius=1.0, dmin=0.5).positions.copy()
    for vertex, expect_ref in ((1, 1), (2, 0)):
        pos = base.copy()
        offs = {0: np.array([0.0, 0, 0]), 1: np.array([0.3, 0, 0]), 2: np.array([0.6, 0, 0])}
        order = [0, 1, 2] if vertex == 1 else [0, 2, 1]
        for w, slot in enumerate(order):
            pos[4 * w:4 * w + 4] += offs[slot] - pos[4 * w]
        for rule, expect in ((0, expect_ref), (1, 1)):
            s = mb.create_mbpol_system(systems.WaterSystem(pos, None, 0, "t"), terms=("threebody",), trimer_rule=rule)
            s.forces[0].setCutoff(0.45)
            ctx = mb.Context(s)
            ctx.setPositions(pos)
            ctx.getState()
            assert ctx.getCounts()[1] == expect, (vertex, rule)
