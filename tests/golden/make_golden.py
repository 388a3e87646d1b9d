"""Generate the golden fixtures under tests/golden/ (run in a checkout with the
reference next to it; the GPU tests only read the committed outputs).

Sources:
  * the reference's own known-answer tests, read as text:
      platforms/reference/tests/TestReferenceMBPolOneBodyForce.cpp:83-113
      platforms/reference/tests/TestReferenceMBPolTwoBodyForce.cpp:99-127
      platforms/reference/tests/TestReferenceMBPolThreeBodyForce.cpp:97-138
      platforms/reference/tests/TestReferenceThreeNeighborList.cpp:42-78
  * the reference's Reference-platform force classes, compiled unmodified by
    oracle/build_ref.sh into oracle/_ref/libmbpol_ref.so, evaluated on seeded
    synthetic systems (mbpol_openmm_plugin_gb300.systems).
Dispersion has no plugin code in the reference (python/mbpol.xml:37-108 builds
an OpenMM CustomNonbondedForce); its values come from the C oracle port.

    python tests/golden/make_golden.py REFERENCE_CHECKOUT [elec|elec_known|pdb|potential|moments|dispersion|box4096|mbpol_xml]
(or "-" for the checkout named by MBPOL_REFERENCE_DIR)
"""
import ctypes
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from mbpol_openmm_plugin_gb300 import systems  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 and sys.argv[1] != "-" else os.environ.get("MBPOL_REFERENCE_DIR", "")
LIB = os.path.join(ROOT, "oracle", "_ref", "libmbpol_ref.so")

VEC3 = r"Vec3\(\s*([-+0-9.eE]+)\s*,\s*([-+0-9.eE]+)\s*,\s*([-+0-9.eE]+)\s*\)"


def parse_test(path, func):
    src = open(path).read()
    i = src.index(func)
    ends = [k for k in (src.find("\nvoid ", i + 10), src.find("\nstatic void ", i + 10), src.find("\nint main", i + 10)) if k > 0]
    body = src[i:min(ends) if ends else len(src)]
    pos, exp = {}, {}
    for m in re.finditer(r"positions\[(\d+)\]\s*=\s*" + VEC3, body):
        pos.setdefault(int(m.group(1)), [float(m.group(k)) for k in (2, 3, 4)])
    for m in re.finditer(r"expectedForces\[(\d+)\]\s*=\s*" + VEC3, body):
        exp.setdefault(int(m.group(1)), [float(m.group(k)) for k in (2, 3, 4)])
    e = re.search(r"expectedEnergy\s*=\s*([-+0-9.eE]+)\s*(\*\s*cal2joule\s*)?;", body)
    n = len(pos)
    return {
        "positions_A": [pos[k] for k in range(n)],
        "expected_gradient_kcal_A": [exp[k] for k in range(len(exp))] if sorted(exp) == list(range(len(exp)))
        else {str(k): v for k, v in exp.items()},
        "expected_energy_kcal": float(e.group(1)),
    }


def lib():
    L = ctypes.CDLL(LIB)
    D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    L.ref_onebody.restype = D
    L.ref_onebody.argtypes = [I, P, I, P, P, P]
    L.ref_twobody.restype = D
    L.ref_twobody.argtypes = [I, P, I, P, P, D, P, P]
    L.ref_threebody.restype = D
    L.ref_threebody.argtypes = [I, P, I, P, P, D, P, P, P, ctypes.c_long]
    L.ref_electrostatics.restype = I
    L.ref_electrostatics.argtypes = [I, P, P, P, P, P, P, P, I, D, D, P, P, D, I, I, P, P, P, P, ctypes.c_char_p, I]
    L.ref_electrostatic_potential.restype = I
    L.ref_electrostatic_potential.argtypes = [I, P, P, P, P, P, P, P, I, D, D, P, P, D, I, I, I, P, P,
                                              ctypes.c_char_p, I]
    L.ref_system_moments.restype = I
    L.ref_system_moments.argtypes = [I, P, P, P, P, P, P, P, I, D, D, P, P, D, I, I, P, P, ctypes.c_char_p, I]
    return L


MW = (0.573293118, 0.213353441, 0.213353441)   # python/mbpol.xml:14
THOLE = [0.4, 0.4, 0.055, 0.626, 0.055]        # python/mbpol.xml:22


def place_m(pos):
    pos = pos.copy()
    for w in range(pos.shape[0] // 4):
        pos[4 * w + 3] = MW[0] * pos[4 * w] + MW[1] * pos[4 * w + 1] + MW[2] * pos[4 * w + 2]
    return pos


def electrostatics(L, pos, box, pme, alpha=0.0, grid=(0, 0, 0), cutoff=0.9, eps=1e-8, maxiter=200):
    """Reference electrostatics for O,H1,H2,M waters with the mbpol.xml
    parameters; M forces are spread back onto O, H1, H2 with the M weights."""
    n = pos.shape[0]
    typ = np.tile([0, 1, 1, 2], n // 4).astype(np.int32)
    q = np.array([-5.1966000e-01, 2.5983000e-01, 2.5983000e-01, 0.0])[typ % 4 if False else [0, 1, 1, 2] * (n // 4)]
    q = np.tile([-5.1966000e-01, 2.5983000e-01, 2.5983000e-01, 0.0], n // 4)
    damp = np.tile([0.00131, 0.000294, 0.000294, 0.00131], n // 4)
    pol = np.tile([0.00131, 0.000294, 0.000294, 0.0], n // 4)
    mol = np.repeat(np.arange(n // 4), 4).astype(np.int32)
    f = np.zeros((n, 3))
    e = ctypes.c_double()
    dip = np.zeros((n, 3))
    it = ctypes.c_int()
    err = ctypes.create_string_buffer(512)
    g = np.array(grid, np.int32)
    b = np.zeros(3) if box is None else np.asarray(box, float)
    th = np.array(THOLE)
    rc = L.ref_electrostatics(n, p(np.ascontiguousarray(pos)), p(q), p(mol), p(typ), p(damp), p(pol), p(th),
                              1 if pme else 0, cutoff, alpha, p(g), p(b), eps, maxiter, 1, p(f),
                              ctypes.byref(e), p(dip), ctypes.byref(it), err, 512)
    if rc:
        raise RuntimeError(err.value.decode())
    for w in range(n // 4):
        fm = f[4 * w + 3].copy()
        f[4 * w + 3] = 0
        for k in range(3):
            f[4 * w + k] += MW[k] * fm
    if not np.isfinite(f).all():
        # The reference's PME forces read uninitialised memory
        # (computeReciprocalSpaceInducedDipoleForceAndEnergy sums
        # multipole[0..9] with only [0] set,
        # MBPolReferenceElectrostaticsForce.cpp:2193-2252); its energies do
        # not.  Use the oracle port's forces, which take the missing
        # multipoles as zero (point charges), for these fixtures.
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        f = oracle.electrostatics_forces(pos, box, alpha, grid, eps)
    return e.value, f, dip, it.value


def p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def run_terms(L, pos, waters, box, cut2=0.65, cut3=0.45):
    pos = np.ascontiguousarray(pos, np.float64)
    w = np.ascontiguousarray(waters, np.int32)
    nw, n = w.shape[0], pos.shape[0]
    b = None if box is None else np.ascontiguousarray(box, np.float64)
    out = {}
    f = np.zeros((n, 3))
    out["e1"] = L.ref_onebody(nw, p(w), n, p(pos), p(b), p(f))
    out["f1"] = f
    f = np.zeros((n, 3))
    npairs = ctypes.c_long()
    out["e2"] = L.ref_twobody(nw, p(w), n, p(pos), p(b), cut2, p(f), ctypes.byref(npairs))
    out["f2"] = f
    out["npairs"] = npairs.value
    f = np.zeros((n, 3))
    nt = ctypes.c_long()
    cap = 4000000
    trips = np.zeros((cap, 3), np.int32)
    out["e3"] = L.ref_threebody(nw, p(w), n, p(pos), p(b), cut3, p(f), ctypes.byref(nt), p(trips), cap)
    out["f3"] = f
    out["ntrip"] = nt.value
    t = trips[:nt.value]
    out["trip_hash"] = int(np.sum((t[:, 0].astype(np.int64) * 1000003 + t[:, 1]) * 1000003 + t[:, 2]) % (1 << 61))
    return out


def dispersion_oracle(pos, waters, box, rc):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # noqa: E402
    return oracle.dispersion(pos, waters, box, rc)


def main():
    L = lib()
    tests = os.path.join(REF, "platforms", "reference", "tests")
    known = {
        "onebody_water1": parse_test(os.path.join(tests, "TestReferenceMBPolOneBodyForce.cpp"), "void testOneOneBody"),
        "twobody_water2": parse_test(os.path.join(tests, "TestReferenceMBPolTwoBodyForce.cpp"), "void testTwoBody"),
        "threebody_water3": parse_test(os.path.join(tests, "TestReferenceMBPolThreeBodyForce.cpp"), "void testThreeBody"),
    }
    # trimer chain rule (TestReferenceThreeNeighborList.cpp:42-78): O positions, cutoff, expected count
    src = open(os.path.join(tests, "TestReferenceThreeNeighborList.cpp")).read()
    known["trimer_rule_source"] = "platforms/reference/tests/TestReferenceThreeNeighborList.cpp:42-78"
    known["trimer_rule_excerpt"] = [ln.strip() for ln in src.splitlines()[41:78]]
    with open(os.path.join(HERE, "reference_known_answers.json"), "w") as f:
        json.dump(known, f, indent=1)

    # the known-answer systems through the compiled reference
    res = {}
    for key, nwat in (("onebody_water1", 1), ("twobody_water2", 2), ("threebody_water3", 3)):
        pos = np.array(known[key]["positions_A"]) * 0.1
        w = np.arange(3 * nwat, dtype=np.int32).reshape(-1, 3)
        r = run_terms(L, pos, w, None, cut2=10.0, cut3=10.0)
        res[key] = {"e1": r["e1"], "e2": r["e2"], "e3": r["e3"],
                    "f1": r["f1"].tolist(), "f2": r["f2"].tolist(), "f3": r["f3"].tolist()}
    with open(os.path.join(HERE, "reference_known_answers_oracle.json"), "w") as f:
        json.dump(res, f, indent=1)

    # seeded synthetic systems: O,H1,H2,M per water (M unused by 1B/2B/3B)
    for name, seed in (("cluster14", 0), ("cluster14", 1), ("box256", 0), ("cluster64", 2)):
        ws = systems.cluster(64, seed, radius=8.0, dmin=2.5) if name == "cluster64" else systems.workload(name, seed)
        waters = ws.water_indices()
        r = run_terms(L, ws.positions, waters, ws.box)
        ed, fd = dispersion_oracle(ws.positions, waters, ws.box, 0.9 if ws.box is not None else 1e30)
        np.savez_compressed(os.path.join(HERE, "%s_seed%d.npz" % (name, seed)),
                            positions=ws.positions, box=np.zeros(3) if ws.box is None else ws.box,
                            periodic=ws.box is not None, e1=r["e1"], e2=r["e2"], e3=r["e3"], f1=r["f1"],
                            f2=r["f2"], f3=r["f3"], npairs=r["npairs"], ntrip=r["ntrip"], trip_hash=r["trip_hash"],
                            edisp=ed, fdisp=fd)
        print(name, seed, "e1 %.6f e2 %.6f e3 %.6f edisp %.6f pairs %d trimers %d" % (
            r["e1"], r["e2"], r["e3"], ed, r["npairs"], r["ntrip"]))


def read_pdb(path):
    xyz = []
    for ln in open(path):
        if ln.startswith(("ATOM", "HETATM")):
            xyz.append([float(ln[30:38]), float(ln[38:46]), float(ln[46:54])])
    return np.array(xyz) * 0.1


def main_pdb():
    """Full-model energies of the reference's integration-test configurations
    (python/tests/pdb_files, boxes and expected totals from
    python/tests/TestReferenceMBPolIntegrationTest.py:12-64 and
    TestReferenceMBPol14WaterTest.py:14-22).  PME alpha and grid are explicit
    (OpenMM's rule at the force's default tolerance 1e-4), since the
    reference takes them from OpenMM's calcPMEParameters."""
    L = lib()
    sys.path.insert(0, ROOT)
    from mbpol_openmm_plugin_gb300.plugin import pme_parameters
    pdbdir = os.path.join(REF, "python", "tests", "pdb_files")
    cases = [("water3", "water3.pdb", None, -8.78893485, 0.1), ("water14", "water14.pdb", None, None, None),
             ("water14_pme", "water14.pdb", 1.8, -60.0, 1.0), ("water50_pme", "water50.pdb", 1.8, -244.37507, 1.0),
             ("water256_pme", "water256_integration_test.pdb", 1.93996888399961804, -2270.88890, 20.0)]
    for name, fn, boxL, expected, tol in cases:
        pos = place_m(read_pdb(os.path.join(pdbdir, fn)))
        nw = pos.shape[0] // 4
        waters = np.stack([4 * np.arange(nw), 4 * np.arange(nw) + 1, 4 * np.arange(nw) + 2], 1).astype(np.int32)
        box = None if boxL is None else np.array([boxL] * 3)
        r = run_terms(L, pos, waters, box)
        ed, fd = dispersion_oracle(pos, waters, box, 0.9 if box is not None else 1e30)
        if box is None:
            ee, fe, dip, it = electrostatics(L, pos, None, False, eps=1e-8)
            alpha, grid = 0.0, [0, 0, 0]
        else:
            alpha, grid = pme_parameters(box, 0.9, 1e-4)
            ee, fe, dip, it = electrostatics(L, pos, box, True, alpha=alpha, grid=grid, eps=1e-8)
        etot = r["e1"] + r["e2"] + r["e3"] + ed + ee
        ftot = r["f1"] + r["f2"] + r["f3"] + fd + fe
        np.savez_compressed(os.path.join(HERE, "pdb_%s.npz" % name), positions=pos,
                            box=np.zeros(3) if box is None else box, periodic=box is not None, alpha=alpha,
                            grid=np.array(grid), e1=r["e1"], e2=r["e2"], e3=r["e3"], edisp=ed, eelec=ee,
                            etotal=etot, ftotal=ftot, f1=r["f1"], f2=r["f2"], f3=r["f3"], fdisp=fd, felec=fe,
                            iterations=it, ntrip=r["ntrip"], npairs=r["npairs"],
                            expected_kcal=np.nan if expected is None else expected,
                            expected_tol_kcal=np.nan if tol is None else tol)
        print("%-14s total %.5f kcal/mol (reference test expects %s +- %s); elec %.4f it %d" % (
            name, etot / 4.184, expected, tol, ee / 4.184, it))


def main_elec():
    L = lib()
    tests = os.path.join(REF, "platforms", "reference", "tests")
    known = parse_test(os.path.join(tests, "TestReferenceMBPolElectrostaticsForce.cpp"), "static void testWater3VirtualSite()")
    pos = place_m(np.array(known["positions_A"]) * 0.1)
    e, f, dip, it = electrostatics(L, pos, None, False, eps=1e-7)
    known["oracle_energy_kJ"] = e
    known["oracle_forces_kJ_nm"] = f.tolist()
    known["oracle_iterations"] = it
    known["source"] = "platforms/reference/tests/TestReferenceMBPolElectrostaticsForce.cpp:419-546"
    with open(os.path.join(HERE, "elec_water3_virtualsite.json"), "w") as fh:
        json.dump(known, fh, indent=1)
    print("water3 virtual site: E %.6f kcal/mol (expected %.6f), iterations %d" % (
        e / 4.184, known["expected_energy_kcal"], it))
    sys.path.insert(0, ROOT)
    from mbpol_openmm_plugin_gb300.plugin import pme_parameters
    for name, seed in (("cluster14", 0), ("cluster14", 1), ("box256", 0)):
        ws = systems.workload(name, seed)
        pos = place_m(ws.positions)
        if ws.box is None:
            e, f, dip, it = electrostatics(L, pos, None, False, eps=1e-8)
            alpha, grid = 0.0, [0, 0, 0]
        else:
            alpha, grid = pme_parameters(ws.box, 0.9, 1e-5)
            e, f, dip, it = electrostatics(L, pos, ws.box, True, alpha=alpha, grid=grid, eps=1e-8)
        np.savez_compressed(os.path.join(HERE, "elec_%s_seed%d.npz" % (name, seed)), positions=pos,
                            box=np.zeros(3) if ws.box is None else ws.box, periodic=ws.box is not None,
                            alpha=alpha, grid=np.array(grid), eelec=e, felec=f, dipoles=dip, iterations=it)
        print(name, seed, "Eelec %.6f kJ/mol  iterations %d  alpha %.4f grid %s" % (e, it, alpha, grid))


def potential_points(pos, box, npts, rng, dmin=0.12):
    """Seeded probe points at least dmin nm from every site: in the box, or
    within 0.4 nm of the cluster's extent."""
    lo, hi = (np.zeros(3), np.asarray(box, float)) if box is not None else (pos.min(0) - 0.4, pos.max(0) + 0.4)
    out = []
    while len(out) < npts:
        g = lo + (hi - lo) * rng.random(3)
        d = pos - g
        if box is not None:
            d -= box * np.round(d / box)
        if np.sqrt((d * d).sum(1)).min() >= dmin:
            out.append(g)
    return np.array(out)


def main_potential():
    """getElectrostaticPotential (MBPolReferenceKernels.cpp:261-283) of the
    compiled reference on seeded probe points."""
    L = lib()
    sys.path.insert(0, ROOT)
    from mbpol_openmm_plugin_gb300.plugin import pme_parameters
    for name, seed in (("cluster14", 0), ("box256", 0)):
        ws = systems.workload(name, seed)
        pos = place_m(ws.positions)
        n = pos.shape[0]
        pts = potential_points(pos, ws.box, 64, np.random.default_rng(1000 + seed))
        if ws.box is None:
            alpha, grid, b = 0.0, [0, 0, 0], np.zeros(3)
        else:
            alpha, grid = pme_parameters(ws.box, 0.9, 1e-5)
            b = np.asarray(ws.box, float)
        typ = np.tile([0, 1, 1, 2], n // 4).astype(np.int32)
        q = np.tile([-5.1966000e-01, 2.5983000e-01, 2.5983000e-01, 0.0], n // 4)
        damp = np.tile([0.00131, 0.000294, 0.000294, 0.00131], n // 4)
        pol = np.tile([0.00131, 0.000294, 0.000294, 0.0], n // 4)
        mol = np.repeat(np.arange(n // 4), 4).astype(np.int32)
        out = np.zeros(len(pts))
        err = ctypes.create_string_buffer(512)
        rc = L.ref_electrostatic_potential(n, p(np.ascontiguousarray(pos)), p(q), p(mol), p(typ), p(damp), p(pol),
                                           p(np.array(THOLE)), 0 if ws.box is None else 1, 0.9, alpha,
                                           p(np.array(grid, np.int32)), p(b), 1e-8, 200, 1, len(pts),
                                           p(np.ascontiguousarray(pts)), p(out), err, 512)
        if rc:
            raise RuntimeError(err.value.decode())
        np.savez_compressed(os.path.join(HERE, "potential_%s_seed%d.npz" % (name, seed)), positions=pos,
                            box=b, periodic=ws.box is not None, alpha=alpha, grid=np.array(grid), points=pts,
                            potential=out)
        print(name, seed, "potential range %.4f .. %.4f kJ/mol/e" % (out.min(), out.max()))


def main_dispersion():
    """Dispersion known answers of the reference's own tests
    (python/tests/TestCustomDispersion.py:14-47, 49-83: water3.pdb and
    water_and_ion.pdb, CutoffNonPeriodic at 1000 nm, -6.84471477 and
    -1.306598 kcal/mol, asserted there to 0.01) with the oracle's energy and
    forces (the reference builds this term from python/mbpol.xml:37-108 as an
    OpenMM CustomNonbondedForce, which is not available here)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    pdbdir = os.path.join(REF, "python", "tests", "pdb_files")
    for name, fn, expected in (("water3", "water3.pdb", -6.84471477),
                               ("water_and_ion", "water_and_ion.pdb", -1.306598)):
        pos = read_pdb(os.path.join(pdbdir, fn))
        nw = pos.shape[0] // 4
        pos = place_m(pos)
        waters = np.stack([4 * np.arange(nw), 4 * np.arange(nw) + 1, 4 * np.arange(nw) + 2], 1).astype(np.int32)
        ions = np.arange(4 * nw, pos.shape[0], dtype=np.int32)
        e, f = oracle.dispersion(pos, waters, ions, None, 1e3)
        np.savez_compressed(os.path.join(HERE, "disp_%s.npz" % name), positions=pos, waters=waters, ions=ions,
                            edisp=e, fdisp=f, expected_kcal=expected, expected_tol_kcal=0.01)
        print("%-14s dispersion %.8f kcal/mol (reference test expects %.8f)" % (name, e / 4.184, expected))


def main_moments():
    """getSystemElectrostaticsMoments (MBPolReferenceKernels.cpp:285-303,
    MBPolReferenceElectrostaticsForce.cpp:923-1021) of the compiled
    reference, with the mbpol.xml masses (python/mbpol.xml:3-5)."""
    L = lib()
    sys.path.insert(0, ROOT)
    from mbpol_openmm_plugin_gb300.plugin import pme_parameters
    for name, seed in (("cluster14", 0), ("box256", 0)):
        ws = systems.workload(name, seed)
        pos = place_m(ws.positions)
        n = pos.shape[0]
        if ws.box is None:
            alpha, grid, b = 0.0, [0, 0, 0], np.zeros(3)
        else:
            alpha, grid = pme_parameters(ws.box, 0.9, 1e-5)
            b = np.asarray(ws.box, float)
        typ = np.tile([0, 1, 1, 2], n // 4).astype(np.int32)
        q = np.tile([-5.1966000e-01, 2.5983000e-01, 2.5983000e-01, 0.0], n // 4)
        damp = np.tile([0.00131, 0.000294, 0.000294, 0.00131], n // 4)
        pol = np.tile([0.00131, 0.000294, 0.000294, 0.0], n // 4)
        mol = np.repeat(np.arange(n // 4), 4).astype(np.int32)
        mass = np.tile([15.99943, 1.007947, 1.007947, 0.0], n // 4)
        out = np.zeros(13)
        err = ctypes.create_string_buffer(512)
        rc = L.ref_system_moments(n, p(np.ascontiguousarray(pos)), p(q), p(mol), p(typ), p(damp), p(pol),
                                  p(np.array(THOLE)), 0 if ws.box is None else 1, 0.9, alpha,
                                  p(np.array(grid, np.int32)), p(b), 1e-8, 200, 1, p(mass), p(out), err, 512)
        if rc:
            raise RuntimeError(err.value.decode())
        np.savez_compressed(os.path.join(HERE, "moments_%s_seed%d.npz" % (name, seed)), positions=pos,
                            box=b, periodic=ws.box is not None, alpha=alpha, grid=np.array(grid), masses=mass,
                            moments=out)
        print(name, seed, "moments", np.array2string(out, precision=5))


ELEC_CASES = [
    # (function, M sites, PME, box nm, cutoff, alpha, grid, eps, redistribution, thole, zero polarity)
    ("static void testWater3()", False, False, None, 0.7, 0.0, None, 1e-9, False, [0.4] * 5, False),
    ("static void testWater3PMEHugeBox()", False, True, 50.0, 0.9, 1e-15, [20, 20, 20], 1e-12, False, [0.4] * 5,
     False),
    ("static void testWater3VirtualSitePMEHugeBox()", True, True, 50.0, 10.0, 1e-15, [20, 20, 20], 1e-4, True,
     THOLE, True),
    ("static void testWater3VirtualSitePMESmallBox()", True, True, 1.8, 0.9, None, None, 1e-12, True, [0.4] * 5,
     False),
]


def parse_elec_test(path, func):
    """Positions, expected energy and forces of one electrostatics test, with
    // comments removed (the small-box test lists its forces by push_back)."""
    src = open(path).read()
    i = src.index(func)
    j = min(k for k in (src.find("\nstatic void ", i + 10), src.find("\nint main", i + 10), len(src)) if k > 0)
    body = "\n".join(ln.split("//")[0] for ln in src[i:j].splitlines())
    pos = {}
    for m in re.finditer(r"positions\[(\d+)\]\s*=\s*" + VEC3, body):
        pos.setdefault(int(m.group(1)), [float(m.group(k)) for k in (2, 3, 4)])
    forces = {}
    for m in re.finditer(r"expectedForces\[(\d+)\]\s*=\s*" + VEC3, body):
        forces[int(m.group(1))] = [float(m.group(k)) for k in (2, 3, 4)]
    pushed = [[float(m.group(k)) for k in (1, 2, 3)]
              for m in re.finditer(r"expectedForces\.push_back\(\s*" + VEC3 + r"\s*\)", body)]
    e = re.search(r"expectedEnergy\s*=\s*([-+0-9.eE]+)\s*(\*\s*cal2joule\s*)?;", body)
    tol = re.search(r"double tolerance\s*=\s*([-+0-9.eE]+)\s*;", body)
    n = len(pos)
    if pushed:
        f = pushed[:n]
    else:
        f = [forces.get(k, [0.0, 0.0, 0.0]) for k in range(n)]
    start = src.count("\n", 0, i) + 1
    return {"positions_A": [pos[k] for k in range(n)], "expected_forces_kcal_A": f,
            "expected_energy": float(e.group(1)), "energy_in_kcal": bool(e.group(2)),
            "tolerance": float(tol.group(1)), "source": "platforms/reference/tests/"
            "TestReferenceMBPolElectrostaticsForce.cpp:%d-%d" % (start, src.count("\n", 0, j) + 1)}


def main_elec_whitebox():
    """The white-box known answers of the reference's electrostatics test:
    getAndScaleInverseRs (testGetAndScaleInverseRs, the intramolecular
    O-H case, and testGetAndScaleInverseRsInterMulecolar) and
    computeWaterCharge (testComputeWaterCharge: charges and charge
    derivatives), read from the test source as text.  In both Thole cases
    the test's last argument selects the Thole parameter by index and every
    parameter is 0.4 (the same value for any index).  Expected values use the
    test's own scalings: rrI[5] carries the factor 3, positions and
    derivatives are converted from Angstrom."""
    path = os.path.join(REF, "platforms", "reference", "tests", "TestReferenceMBPolElectrostaticsForce.cpp")
    src = open(path).read()
    num = r"([-+0-9.eE]+(?:\s*\*\s*[0-9.eE+-]+)*)"

    def ev(expr):
        v = 1.0
        for f in expr.split("*"):
            v *= float(f.strip().rstrip("."))
        return v

    def body_of(func):
        i = src.index("static void " + func + "(") if ("static void " + func + "(") in src else src.index(func)
        j = src.find("\nstatic void ", i + 10)
        j2 = src.find("\nclass ", i + 10)
        j = min(k for k in (j, j2, len(src)) if k > 0)
        return i, j, "\n".join(ln.split("//")[0] for ln in src[i:j].splitlines())

    out = {}
    for func in ("testGetAndScaleInverseRs", "testGetAndScaleInverseRsInterMulecolar"):
        i, j, b = body_of(func)
        damp = re.search(r"RealOpenMM damp\s*=\s*([-+0-9.eE]+)", b)
        dampO = re.search(r"RealOpenMM dampO\s*=\s*([-+0-9.eE]+)", b).group(1)
        dampH = re.search(r"RealOpenMM dampH\s*=\s*([-+0-9.eE]+)", b)
        r = re.search(r"RealOpenMM r\s*=\s*" + num + ";", b).group(1)
        call = re.search(r"wrapGetAndScaleInverseRs\(\s*(\w+),\s*(\w+),", b)
        vals = {"dampO": float(dampO), "dampH": float(dampH.group(1)) if dampH else None}
        exp = {int(m.group(2)): ev(m.group(1))
               for m in re.finditer(r"ASSERT_EQUAL_TOL_MOD\(\s*" + num + r"\s*,\s*rrI\[(\d)\]", b)}
        thole = float(re.search(r"tholes\.push_back\(([0-9.]+)\)", b).group(1))
        out[func] = {"r_nm": ev(r), "damp_i": vals[call.group(1)], "damp_j": vals[call.group(2)], "thole": thole,
                     "expected_rr": [exp[k] for k in (1, 3, 5, 7)], "tolerance": 1e-5,
                     "source": "platforms/reference/tests/TestReferenceMBPolElectrostaticsForce.cpp:%d-%d" % (
                         src.count("\n", 0, i) + 1, src.count("\n", 0, j) + 1)}
    i, j, b = body_of("testComputeWaterCharge")
    pos = [[float(m.group(k)) for k in (2, 3, 4)] for m in re.finditer(r"positions\[(\d+)\]\s*=\s*" + VEC3, b)]
    q = {m.group(2): float(m.group(1)) for m in re.finditer(
        r"ASSERT_EQUAL_TOL_MOD\(\s*([-+0-9.eE]+)\s*,\s*particle(\w+)\.charge", b)}
    der = {int(m.group(1)): [float(m.group(k)) for k in (2, 3, 4)] for m in re.finditer(
        r"expectedChargeDerivatives\[(\d+)\]\s*=\s*" + VEC3, b)}
    out["testComputeWaterCharge"] = {
        "positions_nm": [[0.1 * v for v in p] for p in pos[:3]],
        "charges": [q["O"], q["H1"], q["H2"], q["M"]], "charge_tolerance": 1e-5,
        # rows: particle H1 (0-2), H2 (3-5), O (6-8); each the charge of H1, H2, M; x10 to e/nm
        "derivatives_by_particle": {"H1": [[10 * v for v in der[k]] for k in range(0, 3)],
                                    "H2": [[10 * v for v in der[k]] for k in range(3, 6)],
                                    "O": [[10 * v for v in der[k]] for k in range(6, 9)]},
        "derivative_tolerance": 1e-6,
        "source": "platforms/reference/tests/TestReferenceMBPolElectrostaticsForce.cpp:%d-%d" % (
            src.count("\n", 0, i) + 1, src.count("\n", 0, j) + 1)}
    with open(os.path.join(HERE, "elec_whitebox.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print(json.dumps(out, indent=1)[:1500])


def main_elec_known():
    """The electrostatics known answers of the reference's own tests: water3
    without M sites (NoCutoff and the PME huge box with alpha -> 0), the PME
    huge box with M sites, charge redistribution and zero polarisabilities,
    and the 1.8 nm PME box (alpha and grid from OpenMM's rule at Ewald
    tolerance 1e-3).  Each with the compiled reference's energy and forces
    at the same settings."""
    L = lib()
    sys.path.insert(0, ROOT)
    from mbpol_openmm_plugin_gb300.plugin import pme_parameters
    tests = os.path.join(REF, "platforms", "reference", "tests", "TestReferenceMBPolElectrostaticsForce.cpp")
    out = {}
    for func, msite, pme, boxL, cutoff, alpha, grid, eps, redist, thole, zeropol in ELEC_CASES:
        k = parse_elec_test(tests, func)
        pos = np.array(k["positions_A"]) * 0.1
        if msite:
            pos = place_m(pos)
        n = pos.shape[0]
        K = 4 if msite else 3
        if pme and alpha is None:
            alpha, grid = pme_parameters(np.array([boxL] * 3), cutoff, 1e-3)
        typ = np.tile([0, 1, 1, 2][:K], n // K).astype(np.int32)
        q = np.tile([-5.1966000e-01, 2.5983000e-01, 2.5983000e-01, 0.0][:K], n // K)
        damp = np.tile([0.001310, 0.000294, 0.000294, 0.001310][:K], n // K)
        pol = np.zeros(n) if zeropol else np.tile([0.001310, 0.000294, 0.000294, 0.0][:K], n // K)
        mol = np.repeat(np.arange(n // K), K).astype(np.int32)
        f = np.zeros((n, 3))
        e = ctypes.c_double()
        it = ctypes.c_int()
        err = ctypes.create_string_buffer(512)
        b = np.array([boxL] * 3 if pme else [0.0] * 3)
        rc = L.ref_electrostatics(n, p(np.ascontiguousarray(pos)), p(q), p(mol), p(typ), p(damp), p(pol),
                                  p(np.array(thole, float)), 1 if pme else 0, cutoff, float(alpha or 0.0),
                                  p(np.array(grid or [0, 0, 0], np.int32)), p(b), eps, 500, 1 if redist else 0,
                                  p(f), ctypes.byref(e), None, ctypes.byref(it), err, 512)
        if rc:
            raise RuntimeError(err.value.decode())
        if msite:
            for w in range(n // 4):
                fm = f[4 * w + 3].copy()
                f[4 * w + 3] = 0
                for c in range(3):
                    f[4 * w + c] += MW[c] * fm
        name = func.split()[-1].rstrip("()")
        k.update({"msite": msite, "pme": pme, "box_nm": boxL, "cutoff_nm": cutoff, "alpha": alpha, "grid": grid,
                  "target_epsilon": eps, "charge_redistribution": redist, "thole": thole, "zero_polarity": zeropol,
                  "reference_energy_kJ": e.value, "reference_forces_kJ_nm": f.tolist(),
                  "reference_iterations": it.value})
        out[name] = k
        eexp = k["expected_energy"] * (4.184 if k["energy_in_kcal"] else 1.0)
        print("%-36s expected %.6f kJ/mol, compiled reference %.6f (alpha %s grid %s)" % (
            name, eexp, e.value, alpha, grid))
    with open(os.path.join(HERE, "elec_known_answers.json"), "w") as fh:
        json.dump(out, fh, indent=1)


def main_box4096(frame=None):
    """One frame of the 4096-water benchmark box (systems.workload("box4096",
    0): 49.67 A, jittered 16^3 lattice), all five terms at the benchmark's
    settings: cutoffs 0.65 / 0.45 nm, PME rc 0.9 nm, Ewald tolerance 1e-5
    (alpha and grid explicit), solver threshold 1e-8 D.  Energies of the
    one-, two- and three-body and electrostatics terms come from the
    compiled reference; forces, dipoles and dispersion from the oracle port
    (the reference's PME forces are not finite, see electrostatics() above),
    which agrees with the reference's energies to ~1e-13.

    `frame`: an .npz with `positions` (and `steps`) of the same box after MD
    (written by the GPU MD driver from the lattice, NVE from 300 K
    Maxwell-Boltzmann velocities); the fixture is then box4096_md<steps>.npz.
    Its total energy does not nearly cancel as the lattice frame's does."""
    L = lib()
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from mbpol_openmm_plugin_gb300.plugin import pme_parameters
    ws = systems.workload("box4096", 0)
    out_name = "box4096_seed0.npz"
    if frame is not None:
        fr = np.load(frame)
        ws.positions = np.asarray(fr["positions"], np.float64)
        out_name = "box4096_md%d.npz" % int(fr["steps"])
    pos = place_m(ws.positions)
    nw = pos.shape[0] // 4
    waters = np.stack([4 * np.arange(nw), 4 * np.arange(nw) + 1, 4 * np.arange(nw) + 2], 1).astype(np.int32)
    alpha, grid = pme_parameters(ws.box, 0.9, 1e-5)
    port = oracle.full_model(pos, ws.box, alpha=alpha, grid=grid, eps=1e-8)
    print("port: e1 %.6f e2 %.6f e3 %.6f edisp %.6f eelec %.6f it %d" % (
        port["e1"], port["e2"], port["e3"], port["edisp"], port["eelec"], port["iterations"]), flush=True)
    r = run_terms(L, pos, waters, ws.box)
    ee, _, dip, it = electrostatics(L, pos, ws.box, True, alpha=alpha, grid=grid, eps=1e-8)
    etot = r["e1"] + r["e2"] + r["e3"] + port["edisp"] + ee
    np.savez_compressed(os.path.join(HERE, out_name), positions=pos, box=ws.box, periodic=True,
                        alpha=alpha, grid=np.array(grid), e1=r["e1"], e2=r["e2"], e3=r["e3"], edisp=port["edisp"],
                        eelec=ee, etotal=etot, ftotal=port["ftotal"], dipoles=port["dipoles"],
                        iterations=it, npairs=r["npairs"], ntrip=r["ntrip"], trip_hash=r["trip_hash"],
                        port_energies=np.array([port["e1"], port["e2"], port["e3"], port["edisp"], port["eelec"]]),
                        port_iterations=port["iterations"])
    print("%s: reference e1 %.6f e2 %.6f e3 %.6f eelec %.6f (it %d), total %.6f kJ/mol; pairs %d trimers %d" % (
        out_name, r["e1"], r["e2"], r["e3"], ee, it, etot, r["npairs"], r["ntrip"]))


def main_mbpol_xml():
    """The parameters of the reference's python/mbpol.xml as this package's
    loader reads them (types, masses, the four MBPol elements, the C6/d6
    tables of the dispersion script, the residue template), so that the CPU
    tests check the built-in copy against them without the checkout."""
    sys.path.insert(0, ROOT)
    import mbpol_openmm_plugin_gb300 as mb
    ff = mb.ForceField(os.path.join(REF, "python", "mbpol.xml"))
    out = {"thole": list(ff.thole), "elec": ff.elec, "masses": ff.masses, "cutoff2": ff.cutoff2,
           "cutoff3": ff.cutoff3, "c6": np.asarray(ff.c6).tolist(), "d6": np.asarray(ff.d6).tolist(),
           "templates": ff.templates, "elements": ff.elements, "source": "python/mbpol.xml"}
    with open(os.path.join(HERE, "mbpol_xml_params.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote mbpol_xml_params.json")


if __name__ == "__main__":
    if not REF or not os.path.isdir(REF):
        sys.exit("usage: make_golden.py REFERENCE_CHECKOUT [part] (or '-' with MBPOL_REFERENCE_DIR set)")
    if len(sys.argv) > 2 and sys.argv[2] == "mbpol_xml":
        main_mbpol_xml()
    elif len(sys.argv) > 2 and sys.argv[2] == "box4096":
        main_box4096(sys.argv[3] if len(sys.argv) > 3 else None)
    elif len(sys.argv) > 2 and sys.argv[2] == "elec_known":
        main_elec_known()
    elif len(sys.argv) > 2 and sys.argv[2] == "elec_whitebox":
        main_elec_whitebox()
    elif len(sys.argv) > 2 and sys.argv[2] == "elec":
        main_elec()
    elif len(sys.argv) > 2 and sys.argv[2] == "potential":
        main_potential()
    elif len(sys.argv) > 2 and sys.argv[2] == "pdb":
        main_pdb()
    elif len(sys.argv) > 2 and sys.argv[2] == "moments":
        main_moments()
    elif len(sys.argv) > 2 and sys.argv[2] == "dispersion":
        main_dispersion()
    else:
        main()
        main_elec()
        main_pdb()
        main_potential()
        main_moments()
        main_dispersion()
        main_elec_known()
