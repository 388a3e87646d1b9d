"""CPU: the benchmark line's roofline arithmetic (bench.py), on made-up
kernel timings.  The roofline reports the top kernel of the step's launch
list, the three-body tensor kernel, even when the two-body walk's event time
inside the step is the longer one (it then shares its SMs with the solver);
the walk is reported beside it on the FP32 pipe."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _kern(**ms_per_launch):
    names = ["poly2b", "poly3b", "elec_fixed_field", "elec_induced_update", "elec_pme_dipoles",
             "elec_energy_forces", "elec_direct_field"]
    k = {n: {"total_ms": 0.0, "launches": 0} for n in names}
    for n, (ms, launches) in ms_per_launch.items():
        k[n] = {"total_ms": ms * launches, "launches": launches}
    return k


def test_tensor_work_per_trimer(bench):
    # 239 S blocks x 4 MMAs of 2 * 128 * 64 * 16 flop, per 128 trimers
    assert bench.tc_flop_per_trimer() == pytest.approx(239 * 4 * 2 * 128 * 64 * 16 / 128)


def test_roofline_reports_tensor_kernel_with_walk_beside_it(bench):
    counts = [66450, 174309, 1818204, 16]
    kern = _kern(poly2b=(2.13, 10), poly3b=(2.05, 10), elec_direct_field=(0.09, 160), elec_pme_dipoles=(0.2, 160))
    roof, mem = bench.rooflines(kern, counts, [125, 125, 125], 16384, {"sm_mhz": 2070.0})
    assert roof["kernel"] == "poly3b" and roof["bound"] == "tensor"
    tc = counts[1] * bench.tc_flop_per_trimer() / (2.05e-3) / 1e12
    assert roof["achieved"] == pytest.approx(tc)
    assert roof["frac"] == pytest.approx(roof["achieved"] / roof["peak"])
    walk = roof["two_body_walk"]
    assert walk["kernel"] == "poly2b" and walk["bound"] == "fp32"
    assert walk["achieved"] == pytest.approx(counts[0] * bench.ALGO_FLOP_PER_UNIT["poly2b"] / 2.13e-3 / 1e12)
    assert set(mem) == {"induced_direct_field", "pme_dipole_pass"}
    for m in mem.values():
        assert m["bound"] == "hbm" and m["frac"] == pytest.approx(m["achieved"] / m["peak"])


def test_roofline_without_tensor_kernel_reports_walk(bench):
    kern = _kern(poly2b=(1.7, 5))
    roof, _ = bench.rooflines(kern, [66450, 0, 0, 0], None, 16384, {"sm_mhz": 2070.0})
    assert roof["kernel"] == "poly2b" and roof["bound"] == "fp32"
    assert "two_body_walk" not in roof
