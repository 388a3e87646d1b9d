"""CPU: the tensor-core tables of the three-body polynomial
(codegen/gen_poly_tc.py) reproduce the reference polynomial.

The shifted quadratic form, summed from its three fp16 pieces in FP64,
against the unshifted monomials of the basis extracted from
platforms/reference/src/poly-3b-v2x.cpp (value and gradient), on seeded
trimers of a 14-water cluster and of the 256-water box; and the A-fragment
packing against the PTX register layout of mma.m16n8k16."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from mbpol_openmm_plugin_gb300 import systems
from mbpol_openmm_plugin_gb300.codegen import choose_shift, gen_poly_tc


@pytest.fixture(scope="module")
def tables():
    return gen_poly_tc.build("poly3b")


def _samples(name, n):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    ws = systems.WaterSystem(d["positions"], d["box"] if bool(d["periodic"]) else None, 0, name)
    return choose_shift.threebody_samples(ws, maxn=n)


@pytest.mark.parametrize("name", ["cluster14_seed0", "box256_seed0"])
def test_quadratic_form_matches_polynomial(tables, name):
    X = _samples(name, 300)
    E, G = gen_poly_tc.evaluate(tables, X)
    E0, G0 = gen_poly_tc.trie_eval("poly3b", X)
    # three fp16 pieces hold the scaled rows of S to ~2^-33 of their maxima
    assert np.abs(E - E0).max() <= 1e-8 * max(1.0, np.abs(E0).max())
    assert np.abs(G - G0).max() <= 1e-8 * np.abs(G0).max()


def test_fragment_layout(tables):
    """lane l = 4g + q holds rows g, g+8 and columns 2q, 2q+1, 2q+8, 2q+9 of
    each kept 16x16 tile, lower column in the lower half of each register."""
    t = tables
    frag = t.frag.reshape(-1, 3, 32, 4)
    e = 0
    for i, rt in enumerate(t.rt_id):
        for e in range(t.rt_entry[i], t.rt_entry[i + 1]):
            kt = t.ent_kt[e]
            for p in range(3):
                tile = t.pieces[p][rt * 16:rt * 16 + 16, kt * 16:kt * 16 + 16].view(np.uint16)
                for lane in (0, 5, 31):
                    g, q = lane >> 2, lane & 3
                    want = [(g, 2 * q), (g + 8, 2 * q), (g, 2 * q + 8), (g + 8, 2 * q + 8)]
                    for r, (row, col) in enumerate(want):
                        v = int(frag[e, p, lane, r])
                        assert v & 0xFFFF == tile[row, col] and v >> 16 == tile[row, col + 1]
            if e > 40:
                return


def test_every_row_tile_is_dealt_once(tables):
    t = tables
    assert sorted(t.rt_id.tolist()) == list(range(t.npad // 16))
    assert t.warp_begin[0] == 0 and t.warp_begin[-1] == len(t.rt_id)
    assert t.rt_entry[-1] == len(t.ent_kt) == int(t.occ.sum())
