"""CPU: the committed fixtures reproduce the reference's own known answers
(TestReferenceMBPol{One,Two,Three}BodyForce.cpp), so the compiled reference
that produced them is pinned."""
import json
import os

import numpy as np

from conftest import GOLDEN

KCAL = 4.184


def load():
    known = json.load(open(os.path.join(GOLDEN, "reference_known_answers.json")))
    got = json.load(open(os.path.join(GOLDEN, "reference_known_answers_oracle.json")))
    return known, got


def test_onebody_known_answer():
    known, got = load()
    k, g = known["onebody_water1"], got["onebody_water1"]
    assert abs(g["e1"] / KCAL - k["expected_energy_kcal"]) < 1e-4
    f = np.array(g["f1"]) / (KCAL * 10)
    assert np.allclose(f, -np.array(k["expected_gradient_kcal_A"]), atol=1e-4)


def test_twobody_known_answer():
    known, got = load()
    k, g = known["twobody_water2"], got["twobody_water2"]
    assert abs(g["e2"] / KCAL - k["expected_energy_kcal"]) < 1e-3
    f = np.array(g["f2"]) / (KCAL * 10)
    assert np.allclose(f, -np.array(k["expected_gradient_kcal_A"]), atol=1e-3)


def test_threebody_known_answer():
    known, got = load()
    k, g = known["threebody_water3"], got["threebody_water3"]
    assert abs(g["e3"] / KCAL - k["expected_energy_kcal"]) < 1e-3
    f = np.array(g["f3"]) / (KCAL * 10)
    assert np.allclose(f, -np.array(k["expected_gradient_kcal_A"]), atol=1e-3)


def test_fixture_files_present():
    for name in ("cluster14_seed0", "cluster14_seed1", "box256_seed0", "cluster64_seed2"):
        d = np.load(os.path.join(GOLDEN, name + ".npz"))
        assert d["positions"].shape[1] == 3
        assert np.isfinite(d["f2"]).all() and np.isfinite(d["f3"]).all()
