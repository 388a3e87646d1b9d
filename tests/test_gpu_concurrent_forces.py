"""GPU: the five terms run on concurrent streams and add into one FP64 force
array; repeated evaluations of all terms at the same positions, in one
context and in fresh contexts, must agree with each other and with the sum
of the terms evaluated one at a time to the FP64 atomics' summation order.
(A force kernel that added with a plain read-modify-write while another
stream's atomics wrote the same particles lost updates: 1e2 kJ/mol/nm.)"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import _capi, systems

pytestmark = pytest.mark.gpu
MW = np.array([0.573293118, 0.213353441, 0.213353441])


@pytest.mark.parametrize("name", ["cluster14_seed0", "box256_seed0"])
def test_all_terms_equal_sum_of_single_terms(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    pos = d["positions"].copy()
    pos[3::4] = MW[0] * pos[0::4] + MW[1] * pos[1::4] + MW[2] * pos[2::4]
    box = d["box"] if bool(d["periodic"]) else None
    ws = systems.WaterSystem(pos, box, 0, name)
    lib = _capi.load()
    boxc = None if box is None else np.ascontiguousarray(box, np.float64)

    def evaluate(ctx, mask):
        f = np.zeros_like(pos)
        e = np.zeros(5)
        _capi.check(lib.mbpol_set_positions(ctx._h, _capi.ptr(np.ascontiguousarray(pos)), _capi.ptr(boxc)))
        _capi.check(lib.mbpol_compute(ctx._h, mask, _capi.ptr(e), _capi.ptr(f)))
        return f

    ctx = mb.Context(mb.create_mbpol_system(ws))
    ctx.setPositions(pos)
    ctx._build()
    single = sum(evaluate(ctx, 1 << t) for t in range(5))
    scale = np.abs(single).max()
    worst = 0.0
    for trial in range(3):
        c = ctx if trial == 0 else mb.Context(mb.create_mbpol_system(ws))
        if trial:
            c.setPositions(pos)
            c._build()
        for _ in range(3):
            worst = max(worst, np.abs(evaluate(c, 0x1F) - single).max() / scale)
    print(name, "all terms vs sum of single terms: max relative force difference %.1e" % worst)
    assert worst <= 1e-9
