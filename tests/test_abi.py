"""CPU tests of the C ABI: the library builds for sm_103a, loads, exports
every symbol include/rast_gb300.h declares, and the ctypes mirrors of its
structs have the C compiler's layout.  No compute call is made."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from jaxrenderer_gb300 import _build, _lib

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = []
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(rast_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "rast_render_plain" in names
    for n in names:
        assert hasattr(lib, n), n
    bound = {p[0] for p in _lib.PROTOTYPES}
    assert set(names) == bound, set(names) ^ bound


def test_host_only_entry_points(lib):
    assert lib.rast_abi_version() == _lib.ABI_VERSION == 6
    assert lib.rast_error_string(0) == b"ok"
    assert lib.rast_error_string(6) == b"tile bin capacity exceeded"
    job = _lib.RastJob()
    job.shader = 99
    assert lib.rast_validate_job(ctypes.byref(job)) == 1
    job.shader = 0
    job.width, job.height, job.n_verts, job.n_faces = 4, 4, 3, 1
    assert lib.rast_validate_job(ctypes.byref(job)) == 0
    job.shader = 5  # phong_reflection without textures
    assert lib.rast_validate_job(ctypes.byref(job)) == 1
    assert lib.rast_render_plain(None, None, 0, None) == 1
    assert lib.rast_backward_mse(None, None, 1.0, None, None, None, 0, None) == 1


def _c_layout(tmp_path, struct, fields):
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{ROOT / "include" / "rast_gb300.h"}"',
             "int main(void) {", f'printf("size %zu\\n", sizeof({struct}));']
    for f in fields:
        lines.append(f'printf("{f} %zu\\n", offsetof({struct}, {f}));')
    lines += ["return 0;", "}"]
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}


@pytest.mark.parametrize("struct", ["RastJob", "RastPools", "RastBatch", "RastMesh", "RastInstance", "RastMergeBatch",
                                    "RastTiledConfig", "RastTiledStats", "RastGradPools"])
def test_struct_layout_matches_c(tmp_path, struct):
    cls = getattr(_lib, struct)
    names = [f[0] for f in cls._fields_]
    c = _c_layout(tmp_path, struct, names)
    assert c["size"] == ctypes.sizeof(cls)
    for n in names:
        assert c[n] == getattr(cls, n).offset, n


def test_tile_shapes_without_a_kernel_are_refused_before_any_size_arithmetic(lib):
    """Invalid RastTiledConfig shapes return a status (no division by a zero
    tile side); every call here returns before touching the device."""
    b = _lib.RastBatch()
    b.jobs = 256  # never dereferenced: the shape check comes first
    b.n_jobs, b.max_width, b.max_height = 1, 16, 16
    stats = _lib.RastTiledStats()
    fake_ws = ctypes.c_void_p(256)
    for tw, th in ((0, 0), (0, 8), (8, 0), (-8, 8), (7, 8), (64, 64)):
        cfg = _lib.RastTiledConfig(tw, th, 0)
        assert lib.rast_tiled_workspace_bytes(ctypes.byref(b), ctypes.byref(cfg)) == 0
        assert lib.rast_tiled_stats(ctypes.byref(b), ctypes.byref(cfg), fake_ws, None, ctypes.byref(stats)) == 1
        assert lib.rast_render_tiled(ctypes.byref(b), ctypes.byref(cfg), fake_ws, 1 << 20, None) == 1
        assert lib.rast_render_tiled_static(ctypes.byref(b), ctypes.byref(cfg), None) == 1
    for tw, th in ((16, 8), (32, 8), (8, 4)):  # two warps per tile: 8x8, 8x16 and 16x16 tiles only
        cfg = _lib.RastTiledConfig(tw, th, 0, 0, 2)
        assert lib.rast_tiled_workspace_bytes(ctypes.byref(b), ctypes.byref(cfg)) == 0
        assert lib.rast_render_tiled(ctypes.byref(b), ctypes.byref(cfg), fake_ws, 1 << 20, None) == 1
    assert lib.rast_tiled_workspace_bytes(ctypes.byref(b), ctypes.byref(_lib.RastTiledConfig(8, 16, 0, 0, 1))) == 0
    assert lib.rast_autotune(None, None, ctypes.byref(_lib.RastTiledConfig())) == 1  # no batch: refused on the host
    b.max_layers = 2  # layered batches have kernels for 8x8, 16x8, 8x4 and 4x8 only (and the two-warp tiles)
    cfg = _lib.RastTiledConfig(16, 16, 0)
    assert lib.rast_tiled_workspace_bytes(ctypes.byref(b), ctypes.byref(cfg)) == 0
    assert lib.rast_render_tiled_static(ctypes.byref(b), ctypes.byref(cfg), None) == 4
    assert lib.rast_tiled_workspace_bytes(ctypes.byref(b), ctypes.byref(_lib.RastTiledConfig(16, 16, 0, 0, 2))) > 0
