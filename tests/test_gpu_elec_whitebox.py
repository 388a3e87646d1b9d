"""GPU: the device functions of the electrostatics kernels against the
reference's own white-box known answers (tests/golden/elec_whitebox.json from
platforms/reference/tests/TestReferenceMBPolElectrostaticsForce.cpp:80-131
getAndScaleInverseRs and :326-417 computeWaterCharge), through the C-ABI
probes mbpol_probe_thole_inverse_rs / mbpol_probe_water_charges, at the
test's tolerances (rrI and charges 1e-5 relative to max(|expected|, 1),
derivatives 1e-6), and against the oracle: the Thole factors are FP32 in the
kernels (bar 2e-6 relative to the oracle), the charges FP64 (1e-12)."""
import ctypes
import json
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN
from mbpol_openmm_plugin_gb300 import _capi

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import oracle  # noqa: E402

pytestmark = pytest.mark.gpu
WB = json.load(open(os.path.join(GOLDEN, "elec_whitebox.json")))


def close(expected, found, tol):
    return abs(expected - found) / max(abs(expected), 1.0) <= tol


@pytest.mark.parametrize("case", ["testGetAndScaleInverseRs", "testGetAndScaleInverseRsInterMulecolar"])
def test_device_thole_scaled_inverse_rs(case):
    lib = _capi.load()
    c = WB[case]
    rr = np.zeros(4)
    _capi.check(lib.mbpol_probe_thole_inverse_rs(c["r_nm"], c["damp_i"], c["damp_j"], c["thole"], _capi.ptr(rr)))
    ref = oracle.probe_thole(c["r_nm"], c["damp_i"], c["damp_j"], c["thole"])
    print(case, "device", rr, "expected", c["expected_rr"], "oracle rel", np.abs(rr - ref) / np.abs(ref))
    for e, f in zip(c["expected_rr"], rr):
        assert close(e, f, c["tolerance"])
    assert np.all(np.abs(rr - ref) <= 2e-6 * np.abs(ref))


def test_device_water_charges():
    lib = _capi.load()
    c = WB["testComputeWaterCharge"]
    pos = np.ascontiguousarray(np.array(c["positions_nm"]).reshape(-1))
    q, d = np.zeros(4), np.zeros(27)
    _capi.check(lib.mbpol_probe_water_charges(_capi.ptr(pos), _capi.ptr(q), _capi.ptr(d)))
    d = d.reshape(3, 3, 3)
    qo, do = oracle.probe_water_charges(np.array(c["positions_nm"]))
    print("device charges", q, "expected", c["charges"])
    for e, f in zip(c["charges"], q):
        assert close(e, f, c["charge_tolerance"])
    for name, row in (("O", 0), ("H1", 1), ("H2", 2)):
        exp = np.array(c["derivatives_by_particle"][name])
        assert np.all(np.abs(exp - d[row]) / np.maximum(np.abs(exp), 1.0) <= c["derivative_tolerance"])
    assert np.abs(q - qo).max() <= 1e-12 and np.abs(d - do).max() <= 1e-12


def test_probe_argument_checks():
    lib = _capi.load()
    rr = np.zeros(4)
    assert lib.mbpol_probe_thole_inverse_rs(0.0, 0.001, 0.001, 0.4, _capi.ptr(rr)) == 1
    assert lib.mbpol_probe_water_charges(None, _capi.ptr(rr), _capi.ptr(rr)) == 1
