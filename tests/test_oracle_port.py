"""CPU: the oracle's C port (oracle/mbpol_oracle*.c) against the golden
fixtures produced by the reference's own Reference-platform code (compiled
unmodified, oracle/build_ref.sh) and against the reference's known answers.
This pins the port, which is the checker on machines where the reference
cannot be built."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms

oracle = pytest.importorskip("oracle")


def _w(nw):
    return np.stack([4 * np.arange(nw), 4 * np.arange(nw) + 1, 4 * np.arange(nw) + 2], 1).astype(np.int32)


def P(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


@pytest.mark.parametrize("name", ["cluster14_seed0", "cluster14_seed1", "box256_seed0", "cluster64_seed2"])
def test_port_polyterms_and_dispersion(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    L = oracle.port()
    pos = np.ascontiguousarray(d["positions"])
    box = np.ascontiguousarray(d["box"]) if bool(d["periodic"]) else None
    nw = pos.shape[0] // 4
    w = _w(nw)
    n = pos.shape[0]
    f = np.zeros((n, 3))
    e1 = L.orc_onebody(nw, P(w), P(pos), P(box), P(f))
    assert abs(e1 - float(d["e1"])) <= 1e-10 * abs(float(d["e1"])) and rel_rms(f, d["f1"]) < 1e-10
    f = np.zeros((n, 3))
    npairs = ctypes.c_long()
    e2 = L.orc_twobody(nw, P(w), P(pos), P(box), 0.65, P(f), ctypes.byref(npairs))
    assert abs(e2 - float(d["e2"])) <= 1e-10 * abs(float(d["e2"])) and rel_rms(f, d["f2"]) < 1e-9
    assert npairs.value == int(d["npairs"])
    f = np.zeros((n, 3))
    nt, ns = ctypes.c_long(), ctypes.c_long()
    e3 = L.orc_threebody(nw, P(w), P(pos), P(box), 0.45, 1, P(f), ctypes.byref(nt), ctypes.byref(ns))
    assert abs(e3 - float(d["e3"])) <= 1e-9 * abs(float(d["e3"])) and rel_rms(f, d["f3"]) < 1e-9
    assert nt.value == int(d["ntrip"])
    f = np.zeros((n, 3))
    ed = L.orc_dispersion(nw, P(w), P(pos), P(box), 0.9 if box is not None else 1e30, P(f))
    assert abs(ed - float(d["edisp"])) <= 1e-10 * abs(float(d["edisp"])) and rel_rms(f, d["fdisp"]) < 1e-10


@pytest.mark.parametrize("name", ["water3", "water14", "water14_pme", "water50_pme"])
def test_port_full_model(name):
    """Reference integration configurations (python/tests/pdb_files)."""
    d = np.load(os.path.join(GOLDEN, "pdb_%s.npz" % name))
    periodic = bool(d["periodic"])
    r = oracle.full_model(d["positions"], d["box"] if periodic else None, float(d["alpha"]),
                          [int(v) for v in d["grid"]])
    for k in ("e1", "e2", "e3", "edisp", "eelec"):
        assert abs(r[k] - float(d[k])) <= 1e-9 * max(1.0, abs(float(d[k]))), k
    assert r["iterations"] == int(d["iterations"])
    assert rel_rms(r["ftotal"], d["ftotal"]) < 1e-8
    if not np.isnan(float(d["expected_kcal"])):
        assert abs(r["etotal"] / 4.184 - float(d["expected_kcal"])) <= float(d["expected_tol_kcal"])


def test_port_water3_virtual_site_known_answer():
    """TestReferenceMBPolElectrostaticsForce.cpp:419-546: -15.818784 kcal/mol."""
    import json
    k = json.load(open(os.path.join(GOLDEN, "elec_water3_virtualsite.json")))
    pos = np.array(k["positions_A"]) * 0.1
    for w in range(3):
        pos[4 * w + 3] = 0.573293118 * pos[4 * w] + 0.213353441 * (pos[4 * w + 1] + pos[4 * w + 2])
    r = oracle.full_model(pos, None, eps=1e-7)
    assert abs(r["eelec"] / 4.184 - k["expected_energy_kcal"]) < 1e-4
    assert rel_rms(r["felec"], np.array(k["oracle_forces_kJ_nm"])) < 1e-8


@pytest.mark.parametrize("name", ["potential_cluster14_seed0", "potential_box256_seed0"])
def test_port_electrostatic_potential(name):
    """getElectrostaticPotential (MBPolReferenceElectrostaticsForce.cpp:1023-1085)
    against the compiled reference on seeded probe points."""
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    periodic = bool(d["periodic"])
    out = oracle.electrostatic_potential(d["positions"], d["points"], d["box"] if periodic else None,
                                         float(d["alpha"]), tuple(int(v) for v in d["grid"]))
    ref = d["potential"]
    assert np.max(np.abs(out - ref)) <= 1e-8 * np.max(np.abs(ref))


@pytest.mark.parametrize("name", ["moments_cluster14_seed0", "moments_box256_seed0"])
def test_port_system_moments(name):
    """getSystemElectrostaticsMoments (MBPolReferenceElectrostaticsForce.cpp:
    923-1021) against the compiled reference: charge, dipole and traceless
    quadrupole about the centre of mass."""
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    periodic = bool(d["periodic"])
    out = oracle.system_moments(d["positions"], d["masses"], d["box"] if periodic else None, float(d["alpha"]),
                                tuple(int(v) for v in d["grid"]))
    ref = d["moments"]
    assert np.max(np.abs(out - ref)) <= 1e-10 * np.max(np.abs(ref))


@pytest.mark.parametrize("name", ["disp_water3", "disp_water_and_ion"])
def test_port_dispersion_known_answers(name):
    """Dispersion (python/mbpol.xml:37-108, chloride included) against the
    reference's own known answers (python/tests/TestCustomDispersion.py:14,
    50), at that test's tolerance of 0.01 kcal/mol."""
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    e, f = oracle.dispersion(d["positions"], d["waters"], d["ions"], None, 1e3)
    assert abs(e / 4.184 - float(d["expected_kcal"])) <= float(d["expected_tol_kcal"])
    assert abs(e - float(d["edisp"])) <= 1e-12 * abs(e)
    assert np.allclose(f, d["fdisp"], rtol=0, atol=1e-12)


def test_port_dispersion_ion_forces_match_finite_differences():
    """The port's chloride forces are minus the gradient of its energy
    (central differences on every coordinate of the water-and-ion case)."""
    d = np.load(os.path.join(GOLDEN, "disp_water_and_ion.npz"))
    pos = d["positions"].copy()
    e0, f = oracle.dispersion(pos, d["waters"], d["ions"], None, 1e3)
    h = 1e-6
    for i in (0, 1, 2, 4):
        for k in range(3):
            p = pos.copy()
            p[i, k] += h
            ep, _ = oracle.dispersion(p, d["waters"], d["ions"], None, 1e3)
            p[i, k] -= 2 * h
            em, _ = oracle.dispersion(p, d["waters"], d["ions"], None, 1e3)
            assert abs(-(ep - em) / (2 * h) - f[i, k]) <= 1e-6 * np.abs(f).max()
