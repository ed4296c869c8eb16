"""CPU checks of bench.py's bookkeeping: the compulsory-traffic model behind
the roofline fractions, the per-launch DRAM traffic table it scales, the
peak it divides by and the clock record that decides whether a run stands."""
import json
import os

import pytest

import bench

NNZ = 54.61  # neighbours per particle of the 982,072-particle cylinder


def test_step_roofline_matches_the_compulsory_traffic_model():
    """Per particle-step at 54.61 neighbours: 1,611 B for the mixed form's
    four step kernels and 1,539 B plus 11.5 kflop for the plain form's three
    (each gather: its fields once, the state read and written once, 4 B per
    row entry and 4 B of row length)."""
    mixed = bench.step_roofline("mixed", NNZ, 1.0e9, 1000.0)
    fp64 = bench.step_roofline("fp64", NNZ, 1.0e9, 1000.0)
    assert mixed["bytes_per_particle_step"] == pytest.approx(1611.3, abs=0.1)
    assert fp64["bytes_per_particle_step"] == pytest.approx(1539.3, abs=0.1)
    assert fp64["flops_per_particle_step"] == 11495
    # 1e9 particle-steps/s against a 1,000 GB/s peak
    assert mixed["achieved_gbs"] == pytest.approx(1611.3, abs=0.1)
    assert mixed["frac_hbm"] == pytest.approx(1.6113, abs=1e-4)
    assert fp64["frac_fp64"] == pytest.approx(11.495 / bench.FP64_PEAK_TFLOPS, abs=1e-4)
    for k in bench.STEP_KERNELS["mixed"] + bench.STEP_KERNELS["fp64"]:
        assert bench.ALG_BYTES[k](NNZ) > 0


def test_every_step_kernel_has_a_measured_traffic_figure():
    """The roofline's `traffic` scales the committed per-particle DRAM bytes
    of the timed kernel; every kernel that can be the timed one has a line.
    The mixed kernels move within a factor of two of their algorithmic bytes
    (no gross re-reads); the plain gathers also read or write the pair's
    FP64 kernel gradient once per row entry (8 B), which the compulsory
    model leaves out, and sit within 25 % of the model plus that array."""
    table = {}
    with open(os.path.join(bench.ROOT, "profiles", "traffic_per_launch.txt")) as f:
        for line in f:
            parts = line.split()
            if parts and not parts[0].startswith("#"):
                table[parts[0]] = float(parts[1])
    for k in bench.STEP_KERNELS["mixed"]:
        assert k in table, k
        assert 0.5 <= table[k] / bench.ALG_BYTES[k](NNZ) <= 2.0, k
    for k in bench.STEP_KERNELS["fp64"]:
        assert k in table, k
        assert 0.8 <= table[k] / (bench.ALG_BYTES[k](NNZ) + 8 * NNZ) <= 1.25, k


def test_peak_comes_from_the_measured_file():
    path = os.path.join(bench.ROOT, "MEASURED_PEAKS.json")
    peak, kind = bench.measured_peaks()
    if os.path.exists(path):
        assert kind == "measured" and peak == float(json.load(open(path))["hbm_gbs"])
    else:
        assert (peak, kind) == (6800.0, "fallback")


def test_clock_record_names_active_throttle_reasons():
    """Rows as nvidia-smi prints them (index, sm, max sm, power, active mask,
    hw_slowdown, hw_thermal, sw_thermal, sw_power_cap): only "Active" counts,
    the median SM clock is over the samples."""
    cs = bench.ClockSampler(0)
    cs.rows = [["0", "2070", "2070", "900", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"],
               ["0", "1900", "2070", "1400", "0x4", "Not Active", "Not Active", "Not Active", "Active"],
               ["0", "2050", "2070", "1390", "0x4", "Not Active", "Not Active", "Not Active", "Active"]]
    s = cs.summary()
    assert s["sm_mhz"] == 2050.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    cs.rows.append(["0", "1200", "2070", "1000", "0x40", "Not Active", "Active", "Not Active", "Not Active"])
    assert cs.summary()["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert bench.ClockSampler(0).summary()["reasons"] == ["unsampled"]
