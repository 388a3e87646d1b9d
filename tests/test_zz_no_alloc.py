"""GPU: the no-allocation two-body entry point (mbpol_twobody_dimers_noalloc)
against the context entry point (mbpol_compute with the two-body force only)
on the 256-water box fixture, on two calls in a row.  All device buffers are
allocated here (torch), none by the library.  The kernels are the same, so
the only differences are the orders of the FP64 force/energy atomics:
energy relative error <= 1e-12, forces relative RMS error <= 1e-12.

The file name sorts last so the test also runs after every other GPU test
(the per-device set-up then follows the context path's own uploads); it
passes alone as well."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import _capi, systems

pytestmark = pytest.mark.gpu


def host_dimers(pos, box, rc=0.65):
    """O-O minimum-image distance <= rc, i < j (the context's pair rule)."""
    O = pos[0::4]
    d = O[None, :, :] - O[:, None, :]
    d -= box * np.round(d / box)
    r2 = (d * d).sum(-1)
    i, j = np.nonzero(np.triu(r2 <= rc * rc, 1))
    return np.stack([i, j], 1).astype(np.int32)


def test_noalloc_twobody_matches_context_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    d = np.load(os.path.join(GOLDEN, "box256_seed0.npz"))
    pos = np.ascontiguousarray(d["positions"], np.float64)
    box = np.ascontiguousarray(d["box"], np.float64)
    n = pos.shape[0]
    nw = n // 4

    ws = systems.WaterSystem(pos, box, 0, "fixture")
    ctx = mb.Context(mb.create_mbpol_system(ws, terms=("twobody",)))
    ctx.setPositions(pos)
    st = ctx.getState()
    e_ref, f_ref = st.getPotentialEnergy(), st.getForces()

    dimers = host_dimers(pos, box)
    assert dimers.shape[0] == int(d["npairs"])
    waters = np.stack([4 * np.arange(nw), 4 * np.arange(nw) + 1, 4 * np.arange(nw) + 2, 4 * np.arange(nw) + 3],
                      1).astype(np.int32)
    dev = torch.device("cuda:0")
    t_pos = torch.from_numpy(pos).to(dev)
    t_wat = torch.from_numpy(waters).to(dev)
    t_dim = torch.from_numpy(dimers).to(dev)
    lib = _capi.load()
    stream = torch.cuda.current_stream(dev).cuda_stream
    results = []
    for _ in range(2):
        t_f = torch.zeros((n, 3), dtype=torch.float64, device=dev)
        t_e = torch.zeros(1, dtype=torch.float64, device=dev)
        rc = lib.mbpol_twobody_dimers_noalloc(t_pos.data_ptr(), t_wat.data_ptr(), t_dim.data_ptr(),
                                              int(dimers.shape[0]), _capi.ptr(box), t_f.data_ptr(),
                                              t_e.data_ptr(), stream)
        assert rc == 0, lib.mbpol_last_error()
        torch.cuda.synchronize(dev)
        results.append((float(t_e.cpu()[0]), t_f.cpu().numpy()))
    for e, f in results:
        print("noalloc E %.12f ref %.12f rel %.2e | F relrms %.2e" % (e, e_ref, abs(e - e_ref) / abs(e_ref),
                                                                      rel_rms(f, f_ref)))
        assert abs(e - e_ref) <= 1e-12 * abs(e_ref)
        assert rel_rms(f, f_ref) <= 1e-12
    assert abs(results[0][0] - results[1][0]) <= 1e-12 * abs(e_ref)


def test_noalloc_rejects_oversize_and_misaligned_without_launching():
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    dev = torch.device("cuda:0")
    buf = torch.zeros(64, dtype=torch.float64, device=dev)
    wat = torch.zeros(16, dtype=torch.int32, device=dev)
    p = buf.data_ptr()
    assert lib.mbpol_twobody_dimers_noalloc(p, wat.data_ptr(), wat.data_ptr(), _capi.NOALLOC_MAX_DIMERS + 1,
                                            None, p, p, None) == 5
    assert lib.mbpol_twobody_dimers_noalloc(p, wat.data_ptr() + 4, wat.data_ptr(), 1, None, p, p, None) == 1


FIRST_CALL = r"""
import json, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from mbpol_openmm_plugin_gb300 import _capi
d = np.load(sys.argv[2])
pos = np.ascontiguousarray(d["positions"], np.float64)
n = pos.shape[0]; nw = n // 4
O = pos[0::4]
r2 = ((O[None] - O[:, None]) ** 2).sum(-1)
i, j = np.nonzero(np.triu(r2 <= 0.65 ** 2, 1))
dimers = np.stack([i, j], 1).astype(np.int32)
waters = np.stack([4 * np.arange(nw) + k for k in range(4)], 1).astype(np.int32)
dev = torch.device("cuda:0")
t_pos, t_wat, t_dim = (torch.from_numpy(a).to(dev) for a in (pos, waters, dimers))
t_f = torch.zeros((n, 3), dtype=torch.float64, device=dev)
t_e = torch.zeros(1, dtype=torch.float64, device=dev)
lib = _capi.load()
rc = lib.mbpol_twobody_dimers_noalloc(t_pos.data_ptr(), t_wat.data_ptr(), t_dim.data_ptr(), int(dimers.shape[0]),
                                      None, t_f.data_ptr(), t_e.data_ptr(), None)
torch.cuda.synchronize(dev)
np.save(sys.argv[3], t_f.cpu().numpy())
print(json.dumps({"rc": int(rc), "energy": float(t_e.cpu()[0])}))
"""


def test_noalloc_first_call_in_a_fresh_process_without_box(tmp_path):
    """The entry point's own set-up as the first GPU work of a process (no
    context before it), on a cluster with no box (box_nm NULL: non-periodic),
    against a two-body-only context with the non-periodic cutoff method."""
    pytest.importorskip("torch")
    fx = os.path.join(GOLDEN, "cluster64_seed2.npz")
    out = os.path.join(str(tmp_path), "f.npy")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", FIRST_CALL, root, fx, out], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["rc"] == 0
    d = np.load(fx)
    ws = systems.WaterSystem(d["positions"], None, 0, "fixture")
    ctx = mb.Context(mb.create_mbpol_system(ws, terms=("twobody",)))
    ctx.setPositions(d["positions"])
    st = ctx.getState()
    e_ref, f_ref = st.getPotentialEnergy(), st.getForces()
    f = np.load(out)
    print("first call, no box: E %.12f ref %.12f | F relrms %.2e" % (res["energy"], e_ref, rel_rms(f, f_ref)))
    assert abs(res["energy"] - e_ref) <= 1e-12 * abs(e_ref)
    assert rel_rms(f, f_ref) <= 1e-12


def test_noalloc_rejects_a_box_below_twice_the_cutoff():
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    dev = torch.device("cuda:0")
    buf = torch.zeros(64, dtype=torch.float64, device=dev)
    wat = torch.zeros(16, dtype=torch.int32, device=dev)
    p = buf.data_ptr()
    box = np.array([1.2, 1.2, 1.2])
    assert lib.mbpol_twobody_dimers_noalloc(p, wat.data_ptr(), wat.data_ptr(), 1, _capi.ptr(box), p, p,
                                            None) == 4  # MBPOL_ERR_BOX_TOO_SMALL
