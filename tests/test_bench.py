"""bench.py's roofline arithmetic on the CPU: algorithmic bytes, the measured
raster launch counts (applied only to the launch they were measured on) and
the issue-slot ceiling.  No GPU: the device's SM count is faked."""
import types

import pytest
import torch

import bench


@pytest.fixture
def fake_device(monkeypatch):
    monkeypatch.setattr(torch.cuda, "get_device_properties", lambda d: types.SimpleNamespace(multi_processor_count=152))
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)


def test_kernel_bytes_raster_and_shade():
    info = {"F": 1000.0, "P": 5000.0, "E": 300.0, "T": 10.0, "vs": 10, "main": True, "slots": 1,
            "Ptex": 2000.0, "cin": 0.0, "corners": 3000.0}
    assert bench.kernel_bytes("raster_kernel", info, 0) == 1000 * 48 + 300 * 4 + 5000 * 4
    assert bench.kernel_bytes("tiled_shade_kernel", info, 100) == 5000 * (4 + 16) + 2000 + 100 * (64 + 3 * 4 * 10)
    info["slots"] = 4
    assert bench.kernel_bytes("raster_kernel", info, 0) == 1000 * 48 + 300 * 4 + 5000 * 4 * 4
    assert bench.kernel_bytes("no_such_kernel", info, 0) == 0.0


def test_raster_counts_only_for_the_measured_launch():
    main = types.SimpleNamespace(tile_w=8, tile_h=8)
    assert bench.raster_launch_counts(main, {"P": 4096 * 84 * 84.0}) == bench.NCU_RASTER_LAUNCH[(8, 8, 28901376)]
    assert bench.raster_launch_counts(main, {"P": 256 * 84 * 84.0}) is None  # another batch size
    assert bench.raster_launch_counts(types.SimpleNamespace(tile_w=16, tile_h=8), {"P": 4096 * 84 * 84.0}) is None
    assert bench.raster_launch_counts(None, {"P": 1.0}) is None


def test_issue_roofline(fake_device):
    clocks = {"sm_mhz": 2000.0, "sm_max_mhz": 2070.0}
    peak = 152 * 4 * 2000e6
    got = bench.issue_roofline("raster_kernel", {"P": 1.0}, 2.0, clocks, warp_instr=peak * 1e-3, source="test")
    assert got["peak"] == peak
    assert got["frac"] == pytest.approx(0.5)
    per = bench.NCU_WARP_INSTR_PER_UNIT["tiled_shade_kernel"][1]
    got = bench.issue_roofline("tiled_shade_kernel", {"P": 1e6}, 1.0, clocks)
    assert got["achieved"] == pytest.approx(per * 1e6 / 1e-3)
    assert bench.issue_roofline("raster_kernel", {"P": 1.0}, 1.0, clocks) is None  # no per-unit count
    assert bench.issue_roofline("tiled_shade_kernel", {"P": 1.0}, 1.0, {"sm_mhz": None}) is None
