"""bench.py's roofline arithmetic on the CPU: algorithmic bytes, the ncu
per-unit counts (applied only to the pass and tile configuration they were
measured on, and only while the kernels' sources are the ones measured) and
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


def test_ncu_counts_only_for_the_measured_pass_and_config():
    cfg = lambda w, h, wpt=1: types.SimpleNamespace(tile_w=w, tile_h=h, warps_per_tile=wpt)  # noqa: E731
    assert bench.ncu_per_unit("main", "raster_kernel", cfg(8, 8)) == bench.NCU_PER_UNIT[("main", "raster_kernel", 8, 8, 1)]
    assert bench.ncu_per_unit("main", "raster_kernel", cfg(32, 8)) is None  # another tile shape
    assert bench.ncu_per_unit("main", "raster_kernel", cfg(8, 8, 2)) is None  # two warps per tile
    assert bench.ncu_per_unit("shadow", "raster_kernel", cfg(16, 8))[0] == "P"
    assert bench.ncu_per_unit("main", "tiled_shade_kernel", None)[0] == "P"
    assert bench.ncu_per_unit("main", "raster_kernel", None) is None


def test_counts_are_stamped_with_the_forward_sources():
    assert len(bench.NCU_SOURCE_DIGEST) == 16
    assert bench.library_digest() == bench.library_digest(bench.FORWARD_SOURCES)
    assert bench.library_digest(bench.FORWARD_SOURCES[:1]) != bench.library_digest()


def test_issue_roofline(fake_device):
    clocks = {"sm_mhz": 2000.0, "sm_max_mhz": 2070.0}
    peak = 152 * 4 * 2000e6
    got = bench.issue_roofline(2.0, clocks, peak * 1e-3, "test")
    assert got["peak"] == peak
    assert got["frac"] == pytest.approx(0.5)
    assert bench.issue_roofline(1.0, clocks, None, "test") is None
    assert bench.issue_roofline(1.0, {"sm_mhz": None}, 1.0, "test") is None
