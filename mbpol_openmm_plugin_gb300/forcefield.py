"""PDB files and the MB-pol force field file, for the flow users of the
plugin follow with OpenMM (python/tests/TestReferenceMBPolIntegrationTest.py):

    pdb = PDBFile("water14.pdb")
    ff = ForceField("mbpol.xml")            # or ForceField() for the built-in copy
    system = ff.createSystem(pdb.topology, nonbondedMethod=PME, nonbondedCutoff=0.9)
    context = Context(system); context.setPositions(pdb.positions)

ForceField reads the file format of python/mbpol.xml: atom types (masses),
residue templates (the M virtual site's weights), the MBPolElectrostatics /
OneBody / TwoBody / ThreeBody elements, and the C6 and d6 tables of the
dispersion <Script> (python/mbpol.xml:37-108; the script itself is not
executed, its two numeric tables are read).  createSystem builds the forces
as the generators of python/mbpol.py do (the method maps of :46-49, :118-121,
:191-194, :291-293) and the dispersion as the script does, in the same order
(electrostatics, one-, two-, three-body, the centre-of-mass motion remover,
dispersion), so that code removing forces by index keeps working.  Lengths
are plain floats in nm (OpenMM's unit objects are not available)."""
import re
import xml.etree.ElementTree as ET

import numpy as np

from .plugin import (DISP_C6, DISP_D6, MBPOL_2B_CUTOFF, MBPOL_3B_CUTOFF, MBPOL_CHARGE, MBPOL_DAMPING, MBPOL_MASS,
                     MBPOL_POLARITY, MBPOL_THOLE, MBPolDispersionForce, MBPolElectrostaticsForce, MBPolOneBodyForce,
                     MBPolThreeBodyForce, MBPolTwoBodyForce, System, ThreeParticleAverageSite)

# nonbonded methods (openmm.app names)
NoCutoff, CutoffNonPeriodic, CutoffPeriodic, PME = "NoCutoff", "CutoffNonPeriodic", "CutoffPeriodic", "PME"

# type name -> the electrostatics atom type (python/mbpol.py:5-9)
ATOM_TYPES = {"MBPol-O": 0, "MBPol-H": 1, "MBPol-M": 2}


class CMMotionRemover:
    """Placeholder for the force OpenMM's createSystem adds (removeCMMotion);
    the Context ignores it."""

    _no_kernel = True

    def __init__(self, frequency=1):
        self.frequency = int(frequency)
        self._group = 0

    def getFrequency(self):
        return self.frequency

    def setForceGroup(self, g):
        self._group = int(g)

    def getForceGroup(self):
        return self._group


class Atom:
    def __init__(self, index, name, residue, element):
        self.index, self.name, self.residue, self.element = index, name, residue, element


class Residue:
    def __init__(self, index, name, chain_id, res_id):
        self.index, self.name, self.chain_id, self.id = index, name, chain_id, res_id
        self.atoms_ = []

    def atoms(self):
        return iter(self.atoms_)


class Topology:
    def __init__(self):
        self.atoms_ = []
        self.residues_ = []
        self._box = None

    def atoms(self):
        return iter(self.atoms_)

    def residues(self):
        return iter(self.residues_)

    def getNumAtoms(self):
        return len(self.atoms_)

    def getNumResidues(self):
        return len(self.residues_)

    def getUnitCellDimensions(self):
        return None if self._box is None else self._box.copy()

    def setUnitCellDimensions(self, box):
        self._box = None if box is None else np.asarray(box, float).reshape(3).copy()


class PDBFile:
    """ATOM/HETATM and CRYST1 records (fixed columns of the PDB format);
    positions in nm.  A new residue starts where the residue number, name or
    chain changes."""

    def __init__(self, file):
        self.topology = Topology()
        xyz = []
        lines = file.read().splitlines() if hasattr(file, "read") else open(file).read().splitlines()
        last = None
        for ln in lines:
            rec = ln[:6].strip()
            if rec == "CRYST1":
                self.topology.setUnitCellDimensions([float(ln[6:15]) * 0.1, float(ln[15:24]) * 0.1,
                                                     float(ln[24:33]) * 0.1])
            elif rec in ("ATOM", "HETATM"):
                name = ln[12:16].strip()
                resname = ln[17:20].strip()
                chain = ln[21:22]
                resid = ln[22:26].strip()
                key = (resid, resname, chain)
                if key != last:
                    r = Residue(len(self.topology.residues_), resname, chain, resid)
                    self.topology.residues_.append(r)
                    last = key
                element = ln[76:78].strip() if len(ln) >= 78 else ""
                a = Atom(len(self.topology.atoms_), name, self.topology.residues_[-1], element or name[:1])
                self.topology.residues_[-1].atoms_.append(a)
                self.topology.atoms_.append(a)
                xyz.append([float(ln[30:38]) * 0.1, float(ln[38:46]) * 0.1, float(ln[46:54]) * 0.1])
            elif rec in ("END", "ENDMDL"):
                break
        self.positions = np.array(xyz, float).reshape(-1, 3)

    def getPositions(self, asNumpy=True):
        return self.positions.copy()

    @staticmethod
    def writeFile(topology, positions, file):
        """HETATM records (and CRYST1 when the topology has a unit cell) with
        coordinates in Angstrom to 3 decimals, as OpenMM's PDBFile writes."""
        pos = np.asarray(positions, float).reshape(-1, 3) * 10.0
        out = []
        box = topology.getUnitCellDimensions()
        if box is not None:
            out.append("CRYST1%9.3f%9.3f%9.3f  90.00  90.00  90.00 P 1           1" % tuple(box * 10.0))
        for a in topology.atoms():
            r = a.residue
            out.append("HETATM%5d %-4s %3s %1s%4s    %8.3f%8.3f%8.3f  1.00  0.00          %2s" % (
                (a.index + 1) % 100000, a.name if len(a.name) == 4 else " " + a.name, r.name, r.chain_id or " ",
                r.id, pos[a.index, 0], pos[a.index, 1], pos[a.index, 2], a.element))
        out.append("END")
        text = "\n".join(out) + "\n"
        if hasattr(file, "write"):
            file.write(text)
        else:
            with open(file, "w") as fh:
                fh.write(text)


def water_topology(num_waters, num_ions=0, box=None):
    """Topology of num_waters HOH residues (O, H1, H2, M) followed by
    num_ions Cl residues."""
    top = Topology()
    for w in range(num_waters + num_ions):
        ion = w >= num_waters
        r = Residue(w, "Cl" if ion else "HOH", "A", str(w + 1))
        for name, el in ((("Cl", "Cl"),) if ion else (("O", "O"), ("H1", "H"), ("H2", "H"), ("M", ""))):
            a = Atom(len(top.atoms_), name, r, el)
            r.atoms_.append(a)
            top.atoms_.append(a)
        top.residues_.append(r)
    top.setUnitCellDimensions(box)
    return top


def _table(script, name):
    """The numbers of `name = [ ... ]` in the script text (comments dropped)."""
    m = re.search(r"\b%s\s*=\s*\[(.*?)\]" % re.escape(name), script, re.S)
    if not m:
        raise ValueError("no %s table in the force field's script" % name)
    body = "\n".join(ln.split("#", 1)[0] for ln in m.group(1).splitlines())
    vals = [float(v) for v in body.replace("\n", " ").split(",") if v.strip()]
    return np.array(vals, float)


class ForceField:
    """The MB-pol force field: the parameters of python/mbpol.xml, built in
    (no argument) or read from files of that format."""

    def __init__(self, *files):
        # built-in copy (the constants of plugin.py, each citing mbpol.xml)
        self.masses = {"MBPol-O": MBPOL_MASS[0], "MBPol-H": MBPOL_MASS[1], "MBPol-M": MBPOL_MASS[2],
                       "MBPol-Cl": 35.4532}
        self.type_class = {"MBPol-O": "O", "MBPol-H": "H", "MBPol-M": "M", "MBPol-Cl": "CL"}
        self.templates = {"HOH": {"atoms": {"O": "MBPol-O", "H1": "MBPol-H", "H2": "MBPol-H", "M": "MBPol-M"},
                                  "vsite": ("M", ("O", "H1", "H2"), (0.573293118, 0.213353441, 0.213353441))},
                          "Cl": {"atoms": {"Cl": "MBPol-Cl"}, "vsite": None}}
        self.thole = list(MBPOL_THOLE)
        self.elec = {"MBPol-O": (MBPOL_CHARGE[0], MBPOL_DAMPING[0], MBPOL_POLARITY[0]),
                     "MBPol-H": (MBPOL_CHARGE[1], MBPOL_DAMPING[1], MBPOL_POLARITY[1]),
                     "MBPol-M": (MBPOL_CHARGE[2], MBPOL_DAMPING[2], MBPOL_POLARITY[2])}
        self.cutoff2 = MBPOL_2B_CUTOFF
        self.cutoff3 = MBPOL_3B_CUTOFF
        self.c6 = np.array(DISP_C6, float)
        self.d6 = np.array(DISP_D6, float)
        self.elements = {"elec": True, "one": True, "two": True, "three": True, "disp": True}
        if files:
            self.elements = dict.fromkeys(self.elements, False)
            self.templates = {}
            for f in files:
                self._load(f)

    def _load(self, path):
        root = ET.parse(path).getroot()
        for t in root.iter("Type"):
            self.masses[t.get("name")] = float(t.get("mass", "0"))
            self.type_class[t.get("name")] = t.get("class")
        res = root.find("Residues")
        for r in (res.findall("Residue") if res is not None else []):
            atoms = {a.get("name"): a.get("type") for a in r.findall("Atom")}
            names = [a.get("name") for a in r.findall("Atom")]
            vs = None
            for v in r.findall("VirtualSite"):
                if v.get("type") != "average3":
                    raise ValueError("virtual site type %s is not supported" % v.get("type"))
                idx = [int(v.get(k)) for k in ("index", "atom1", "atom2", "atom3")]
                w = tuple(float(v.get(k)) for k in ("weight1", "weight2", "weight3"))
                vs = (names[idx[0]], tuple(names[i] for i in idx[1:]), w)
            self.templates[r.get("name")] = {"atoms": atoms, "vsite": vs}
        e = root.find("MBPolElectrostaticsForce")
        if e is not None:
            self.elements["elec"] = True
            # python/mbpol.py:266-269: five components, dipole-dipole twice
            keys = ["thole-charge-charge", "thole-charge-dipole", "thole-dipole-dipole",
                    "thole-dipole-dipole-singlebond", "thole-dipole-dipole"]
            self.thole = [float(e.get(k)) for k in keys]
            for a in e.findall("Atom"):
                self.elec[a.get("type")] = (float(a.get("charge")), float(a.get("damping-factor")),
                                            float(a.get("polarizability")))
        if root.find("MBPolOneBodyForce") is not None:
            self.elements["one"] = True
        for tag, attr, key in (("MBPolTwoBodyForce", "cutoff2", "two"), ("MBPolThreeBodyForce", "cutoff3", "three")):
            el = root.find(tag)
            if el is not None:
                self.elements[key] = True
                setattr(self, attr, float(el.get("cutoff_nm")))
        s = root.find("Script")
        if s is not None and s.text and "C6table" in s.text:
            self.elements["disp"] = True
            self.c6 = _table(s.text, "C6table")
            self.d6 = _table(s.text, "d6table")
            if self.c6.size != 16 or self.d6.size != 16:
                raise ValueError("the dispersion tables must be 4 x 4")

    def createSystem(self, topology, nonbondedMethod=NoCutoff, nonbondedCutoff=1.0, removeCMMotion=True,
                     ewaldErrorTolerance=None):
        """The System of `topology` (HOH waters with atoms O, H1, H2, M and
        Cl ions), forces in the order ForceField('mbpol.xml') creates them."""
        sys_ = System()
        waters, ions = [], []
        cls = []
        for r in topology.residues():
            tpl = self.templates.get(r.name)
            if tpl is None:
                raise ValueError("no template for residue %s %s" % (r.name, r.id))
            byname = {a.name: a for a in r.atoms()}
            for a in r.atoms():
                t = tpl["atoms"].get(a.name)
                if t is None:
                    raise ValueError("no type for atom %s %s %s" % (a.name, r.name, r.id))
                sys_.addParticle(self.masses[t])
                cls.append(t)
            if tpl["vsite"] is not None:
                site, parents, w = tpl["vsite"]
                sys_.setVirtualSite(byname[site].index,
                                    ThreeParticleAverageSite(*(byname[p].index for p in parents), *w))
            if r.name == "HOH":
                waters.append((byname["O"].index, byname["H1"].index, byname["H2"].index, byname["M"].index))
            elif tpl["atoms"] and all(t == "MBPol-Cl" for t in tpl["atoms"].values()):
                ions.extend(a.index for a in r.atoms())
        periodic = nonbondedMethod in (PME, CutoffPeriodic)
        if periodic:
            box = topology.getUnitCellDimensions()
            if box is None:
                raise ValueError("a periodic method needs the topology's unit cell")
            sys_.setDefaultPeriodicBoxVectors((box[0], 0, 0), (0, box[1], 0), (0, 0, box[2]))
        if nonbondedMethod not in (NoCutoff, CutoffNonPeriodic, CutoffPeriodic, PME):
            raise ValueError("unknown nonbonded method %r" % (nonbondedMethod,))
        w3 = [list(w[:3]) for w in waters]
        if self.elements["elec"]:
            if nonbondedMethod == CutoffPeriodic:
                raise ValueError("Illegal nonbonded method for MBPolElectrostaticsForce")
            f = MBPolElectrostaticsForce()
            f.setCutoffDistance(float(nonbondedCutoff))
            f.setNonbondedMethod(MBPolElectrostaticsForce.PME if nonbondedMethod == PME
                                 else MBPolElectrostaticsForce.NoCutoff)
            f.setTholeParameters(self.thole)
            if ewaldErrorTolerance is not None:
                f.setEwaldErrorTolerance(float(ewaldErrorTolerance))
            for i, w in enumerate(waters):
                for p in w:
                    q, dmp, pol = self.elec[cls[p]]
                    f.addElectrostatics(q, i, ATOM_TYPES[cls[p]], dmp, pol)
            sys_.addForce(f)
        if self.elements["one"]:
            f = MBPolOneBodyForce()
            f.setNonbondedMethod(MBPolOneBodyForce.Periodic if periodic else MBPolOneBodyForce.NonPeriodic)
            for w in w3:
                f.addOneBody(w)
            sys_.addForce(f)
        for key, F, rc in (("two", MBPolTwoBodyForce, self.cutoff2), ("three", MBPolThreeBodyForce, self.cutoff3)):
            if not self.elements[key]:
                continue
            f = F()
            f.setCutoff(rc)
            f.setNonbondedMethod({NoCutoff: F.NoCutoff, CutoffNonPeriodic: F.CutoffNonPeriodic}.get(
                nonbondedMethod, F.CutoffPeriodic))
            for w in w3:
                f.addParticle(w)
            sys_.addForce(f)
        if removeCMMotion:
            sys_.addForce(CMMotionRemover())
        if self.elements["disp"]:
            f = MBPolDispersionForce()
            f.c6 = self.c6.copy()
            f.d6 = self.d6.copy()
            f.setCutoff(float(nonbondedCutoff))
            f.setNonbondedMethod({NoCutoff: MBPolDispersionForce.NoCutoff,
                                  CutoffNonPeriodic: MBPolDispersionForce.CutoffNonPeriodic}.get(
                nonbondedMethod, MBPolDispersionForce.CutoffPeriodic))
            for w in w3:
                f.addParticle(w)
            for i in ions:
                f.addIon(i)
            sys_.addForce(f)
        return sys_
