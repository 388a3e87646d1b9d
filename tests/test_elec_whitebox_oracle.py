"""CPU: the oracle's Thole scale factors and water charges against the
white-box known answers of the reference's own electrostatics test
(tests/golden/elec_whitebox.json, read from
platforms/reference/tests/TestReferenceMBPolElectrostaticsForce.cpp by
make_golden.py elec_whitebox), at that test's tolerances: rrI to 1e-5 and
charges to 1e-5 relative to max(|expected|, 1), charge derivatives to 1e-6."""
import json
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import oracle  # noqa: E402

WB = json.load(open(os.path.join(GOLDEN, "elec_whitebox.json")))


def close(expected, found, tol):
    return abs(expected - found) / max(abs(expected), 1.0) <= tol


@pytest.mark.parametrize("case", ["testGetAndScaleInverseRs", "testGetAndScaleInverseRsInterMulecolar"])
def test_oracle_thole_scaled_inverse_rs(case):
    c = WB[case]
    rr = oracle.probe_thole(c["r_nm"], c["damp_i"], c["damp_j"], c["thole"])
    print(case, rr, c["expected_rr"])
    for e, f in zip(c["expected_rr"], rr):
        assert close(e, f, c["tolerance"])


def test_oracle_water_charges():
    c = WB["testComputeWaterCharge"]
    q, d = oracle.probe_water_charges(np.array(c["positions_nm"]))
    print("charges", q, c["charges"])
    for e, f in zip(c["charges"], q):
        assert close(e, f, c["charge_tolerance"])
    for name, row in (("O", 0), ("H1", 1), ("H2", 2)):
        exp = np.array(c["derivatives_by_particle"][name])
        for s in range(3):
            for k in range(3):
                assert close(exp[s][k], d[row][s][k], c["derivative_tolerance"]), (name, s, k, exp[s][k], d[row][s][k])
