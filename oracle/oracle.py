"""The oracle: FP64 CPU restatement of the MB-pol reference's algorithms.

TEST INFRASTRUCTURE ONLY.  It is imported by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg, as the checker; the product library never
calls it.

  * dispersion (numpy): python/mbpol.xml:37-108 (the CustomNonbondedForce
    expression -C6*tt6/r^6, exclusions: same water or any M site);
  * the other terms: the C port oracle/mbpol_oracle.c, loaded from
    oracle/_port/libmbpol_oracle.so (built by build_port()).
Pinned against the reference's own known-answer tests and against the
reference's Reference-platform code compiled unmodified (oracle/build_ref.sh),
through the fixtures in tests/golden/.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_DIR = os.path.join(HERE, "_port")
PORT_LIB = os.path.join(PORT_DIR, "libmbpol_oracle.so")

# python/mbpol.xml:52-83, classes O=0, H=1
_C6 = {(0, 0): 9.92951990e-4, (0, 1): 3.49345451e-4, (1, 0): 3.49345451e-4, (1, 1): 8.40715638e-5}
_D6 = {(0, 0): 9.29548582e+01, (0, 1): 9.77520243e+01, (1, 0): 9.77520243e+01, (1, 1): 9.40647517e+01}


def dispersion(pos, waters, box, rc):
    """Energy (kJ/mol) and forces (kJ/mol/nm) of the MB-pol dispersion over
    the O/H sites of `waters` (nw x 3 particle indices)."""
    pos = np.asarray(pos, float)
    waters = np.asarray(waters, int)
    f = np.zeros_like(pos)
    e = 0.0
    nw = waters.shape[0]
    cls = np.array([0, 1, 1])
    for i in range(nw):
        for j in range(i + 1, nw):
            for a in range(3):
                for b in range(3):
                    d = pos[waters[j, b]] - pos[waters[i, a]]
                    if box is not None:
                        d = d - box * np.floor(d / box + 0.5)
                    r2 = d @ d
                    if r2 > rc * rc:
                        continue
                    r = np.sqrt(r2)
                    key = (cls[a], cls[b])
                    c6, d6 = _C6[key], _D6[key]
                    x = d6 * r
                    s6 = sum(x ** n / np.math.factorial(n) for n in range(7)) if hasattr(np, "math") else None
                    if s6 is None:
                        import math
                        s6 = sum(x ** n / math.factorial(n) for n in range(7))
                    tt = 1.0 - np.exp(-x) * s6
                    import math
                    dtt = d6 * np.exp(-x) * x ** 6 / math.factorial(6)
                    e += -c6 * tt / r ** 6
                    dEdr = -c6 * (dtt / r ** 6 - 6.0 * tt / r ** 7)
                    fv = -dEdr * d / r
                    f[waters[j, b]] += fv
                    f[waters[i, a]] -= fv
    return e, f


def build_port(force=False):
    """Compile oracle/mbpol_oracle.c into oracle/_port (gcc, plain C)."""
    src = os.path.join(HERE, "mbpol_oracle.c")
    os.makedirs(PORT_DIR, exist_ok=True)
    if not force and os.path.exists(PORT_LIB) and os.path.getmtime(PORT_LIB) >= os.path.getmtime(src):
        return PORT_LIB
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-I", os.path.join(HERE, "gen"),
                           src, "-o", PORT_LIB, "-lm"])
    return PORT_LIB
