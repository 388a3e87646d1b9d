"""Build the MB-pol GB300 library in-tree: mbpol_openmm_plugin_gb300/lib/libmbpol_gb300.so.

Steps (independent ones in parallel):
  1. model tables (one-body PES) -> csrc/gen/model_tables.inc, from data/;
  2. nvcc -c for each csrc/*.cu (sm_103a only), then one shared link with cuFFT.
The polynomial trie tables (csrc/gen/poly*_tables.inc) are generated by
codegen/gen_poly.py and committed; the tensor-core tables of the three-body
polynomial are generated here by codegen/gen_poly_tc.py (a few seconds,
numpy) into _build/poly_tc_tables.cpp and compiled by the host compiler.
Only sm_103a code is produced.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
GEN = os.path.join(CSRC, "gen")
DATA = os.path.join(PKG, "data")
OUT = os.path.join(PKG, "lib")
BUILD = os.path.join(PKG, "_build")
ARCH = "sm_103a"
NVCC = os.environ.get("NVCC", "nvcc")
LIBNAME = "libmbpol_gb300.so"


def run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def gen_model_tables():
    rows = []
    for line in open(os.path.join(DATA, "onebody_tables.txt")):
        if line.startswith("#") or line.startswith("n "):
            continue
        t = line.split()
        rows.append(([float(v) for v in t[:4]], [int(v) for v in t[4:7]]))
    # combined coefficients (MBPolReferenceOneBodyForce.cpp:99-101):
    # c5z = f5z*c5zA + fbasis*cbasis + fcore*ccore + frest*crest
    f5z, fbasis, fcore, frest = 0.999677885, 0.15860145369897, -1.6351695982132, 1.0
    coef = [f5z * c[0] + fbasis * c[1] + fcore * c[2] + frest * c[3] for c, _ in rows]
    out = ["// Generated by build.py from data/onebody_tables.txt. Do not edit.",
           "static const double kOneBodyCoef[245] = {"]
    out += ["    %.17e," % c for c in coef]
    out.append("};")
    out.append("static const unsigned char kOneBodyIdx[3][245] = {")
    for k in range(3):
        out.append("    {" + ",".join(str(ix[k]) for _, ix in rows) + "},")
    out.append("};")
    path = os.path.join(GEN, "model_tables.inc")
    text = "\n".join(out) + "\n"
    if not os.path.exists(path) or open(path).read() != text:
        with open(path, "w") as f:
            f.write(text)


def compile_cu(src):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps += [os.path.join(GEN, f) for f in os.listdir(GEN)]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return obj
    run([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
         "-Xcompiler", "-fPIC", "-I", BUILD, "-I", CSRC, "-c", src, "-o", obj])
    return obj


def gen_tc_tables():
    """codegen/gen_poly_tc.py -> _build/poly_tc_tables.cpp -> object (g++)."""
    src = os.path.join(BUILD, "poly_tc_tables.cpp")
    obj = src + ".o"
    inputs = [os.path.join(PKG, "codegen", f) for f in ("gen_poly_tc.py", "gen_poly.py")]
    inputs += [os.path.join(DATA, "poly3b_%s.txt" % k) for k in ("basis", "coeffs", "shift")]
    inputs.append(os.path.join(CSRC, "poly_tc.h"))
    if not os.path.exists(obj) or any(os.path.getmtime(obj) < os.path.getmtime(f) for f in inputs):
        sys.path.insert(0, os.path.dirname(PKG))
        from mbpol_openmm_plugin_gb300.codegen import gen_poly_tc
        gen_poly_tc.generate(src)
        run([os.environ.get("CXX", "g++"), "-std=c++17", "-O1", "-fPIC", "-I", CSRC, "-c", src, "-o", obj])
    return obj


def build(verbose=True):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(OUT, exist_ok=True)
    gen_model_tables()
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    with ThreadPoolExecutor(max_workers=max(4, os.cpu_count() or 4)) as ex:
        tc = ex.submit(gen_tc_tables)
        objs = list(ex.map(compile_cu, srcs))
        objs.append(tc.result())
    lib = os.path.join(OUT, LIBNAME)
    tmp = lib + ".tmp"
    run([NVCC, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs + ["-lcufft", "-lcudart"])
    os.replace(tmp, lib)
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build()
