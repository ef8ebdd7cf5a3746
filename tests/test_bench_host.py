"""Host-side pieces of bench.py that need no GPU: the clock-sample parser picks
the benchmarked GPU's rows by UUID, not by nvidia-smi's PCI-order index."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

MINE = "GPU-3f0c1a2b-0000-1111-2222-333344445555"
OTHER = "GPU-99999999-aaaa-bbbb-cccc-dddddddddddd"


def _row(uuid, index, sm, smax=2070, hw="Not Active", pc="Not Active"):
    return (f"{uuid}, {index}, {sm}, {smax}, 900.0, 0x0000000000000000, {hw}, Not Active, "
            f"Not Active, {pc}\n")


def test_clock_samples_selected_by_uuid_not_index():
    # this process's GPU is physical index 3 (CUDA ordinal 0 under
    # CUDA_VISIBLE_DEVICES=3); index 0 belongs to someone else and throttles
    lines = []
    for k in range(6):
        lines.append(_row(OTHER, 0, 990, hw="Active"))
        lines.append(_row(MINE, 3, 2070 if k else 345, pc="Active" if k == 2 else "Not Active"))
    out = bench.parse_clock_samples(lines, MINE)
    assert out["samples"] == 6
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]        # not the other GPU's hw_slowdown
    assert out["gpu"] == MINE


def test_clock_samples_without_matching_rows():
    out = bench.parse_clock_samples([_row(OTHER, 0, 2070)], MINE)
    assert out["sm_mhz"] is None and out["reasons"] == ["no samples"]
    # rows of the older query form (no uuid column) are ignored, not misread
    assert bench.parse_clock_samples(["0, 2070, 2070, 900, 0x0, Not Active, Not Active, "
                                      "Not Active, Not Active\n"], MINE)["sm_mhz"] is None


def test_clock_query_fields_in_parser_order():
    fields = bench.CLOCK_QUERY.split(",")
    assert fields[0] == "uuid" and fields[2] == "clocks.sm" and fields[3] == "clocks.max.sm"
    assert fields[6:10] == ["clocks_event_reasons.hw_slowdown",
                            "clocks_event_reasons.hw_thermal_slowdown",
                            "clocks_event_reasons.sw_thermal_slowdown",
                            "clocks_event_reasons.sw_power_cap"]
