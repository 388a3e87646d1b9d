"""GPU: the launch-shape autotuner (mbpol_set_autotune).  On the 256-water
PME box with the three-body term on the tensor cores: 12 evaluations per
repetition visit every candidate shape, the tuner then settles on one of
them, and every shape gives the same energies and forces (the persistent
kernels' arithmetic per unit does not depend on the grid; FP64 force
atomics sum in no fixed order: 1e-12)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import systems

pytestmark = pytest.mark.gpu


def test_autotune_visits_shapes_and_keeps_results():
    d = np.load(os.path.join(GOLDEN, "box256_seed0.npz"))
    ws = systems.WaterSystem(d["positions"], d["box"], 0, "fixture")
    s = mb.create_mbpol_system(ws, terms=("twobody", "threebody"))
    for f in s.forces:
        if isinstance(f, mb.MBPolThreeBodyForce):
            f.setPolynomialEvaluator(f.TensorCores)
    ctx = mb.Context(s)
    ctx.setPositions(d["positions"])
    ref = ctx.getState()
    assert ctx.getLaunchShape() == (52, 24, False)
    ctx.setAutotune(1)
    for i in range(12):
        assert not ctx.getLaunchShape()[2]
        ctx.setPositions(d["positions"])
        st = ctx.getState()
        assert abs(st.getPotentialEnergy() - ref.getPotentialEnergy()) <= 1e-12 * abs(ref.getPotentialEnergy())
        assert rel_rms(st.getForces(), ref.getForces()) <= 1e-12
    tc, walk, tuned = ctx.getLaunchShape()
    print("tuned shape: tensor kernel leaves %d SMs, walks leave %d blocks" % (tc, walk))
    assert tuned and tc in (0, 26, 52, 76) and walk in (0, 48, 96)
    ctx.setLaunchShape(0, 0)
    assert ctx.getLaunchShape() == (0, 0, False)
    ctx.setPositions(d["positions"])
    st = ctx.getState()
    assert abs(st.getPotentialEnergy() - ref.getPotentialEnergy()) <= 1e-12 * abs(ref.getPotentialEnergy())
