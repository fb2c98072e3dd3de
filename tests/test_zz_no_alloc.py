"""rast_render_tiled_static: the tiled renderer without any allocation.

Some callers cannot allocate device memory at the point where they render:
a CUDA-graph capture without a memory pool, a framework callback that
forbids cudaMalloc, a real-time render thread that must not touch the
allocator, or a plugin whose host owns all device memory.  For them the
library offers one entry point that runs the tiled form out of a static
64 MiB device array instead of a caller-provided workspace.  This checks,
through the C ABI, that two calls in a row give exactly what the
workspace entry point gives without moving the device's free memory, that
the call captured into a CUDA graph replays to the same buffers, and that a
batch too large for the array is refused before anything runs.  It sits in a file of its own that pytest
collects last.
"""
import ctypes

import pytest
import torch

from jaxrenderer_gb300 import _lib
from jaxrenderer_gb300.jobs import pack
from tests import scenes

pytestmark = pytest.mark.gpu


def _snapshot(packed):
    return (packed.zbuffer.clone(), packed.canvas.clone(), packed.prim_id.clone())


def _restore(packed, init):
    packed.zbuffer.copy_(init[0])
    packed.canvas.copy_(init[1])
    packed.prim_id.fill_(-7)


def _assert_same(a, b):
    assert torch.equal(a[2], b[2]), "winning-primitive buffers differ"
    assert torch.equal(a[0].view(torch.int32), b[0].view(torch.int32)), "z-buffers differ"
    assert torch.allclose(a[1], b[1], rtol=0, atol=1e-5), "canvases differ"


def test_static_scratch_entry_point_matches_workspace_entry_point(cuda_device):
    lib = _lib.load()
    specs = [scenes.random_job(sh, seed=900 + sh, W=40 + 3 * sh, H=36, F=120) for sh in scenes.ALL_SHADERS]
    bufs = [scenes.initial_buffers(s) for s in specs]
    packed = pack(specs, [b[0] for b in bufs], [b[1] for b in bufs], cuda_device)
    b = packed.batch
    cfg = _lib.RastTiledConfig(8, 8, 0)
    need = lib.rast_tiled_workspace_bytes(ctypes.byref(b), ctypes.byref(cfg))
    assert need <= _lib.STATIC_SCRATCH_BYTES
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    init = _snapshot(packed)

    ws = torch.empty(int(need), dtype=torch.uint8, device=cuda_device)
    assert lib.rast_render_tiled(ctypes.byref(b), ctypes.byref(cfg), ws.data_ptr(), need, stream) == 0
    expected = _snapshot(packed)

    for k in range(2):  # the array keeps the previous call's contents
        _restore(packed, init)
        torch.cuda.synchronize(cuda_device)
        free_before = torch.cuda.mem_get_info(cuda_device)[0]
        assert lib.rast_render_tiled_static(ctypes.byref(b), ctypes.byref(cfg), stream) == 0
        torch.cuda.synchronize(cuda_device)
        if k == 1:  # after the first call's one-time set-up: the device's free memory does not move
            assert torch.cuda.mem_get_info(cuda_device)[0] == free_before
        _assert_same(_snapshot(packed), expected)
    assert (expected[2] >= 0).any()


def test_static_scratch_entry_point_replays_from_a_cuda_graph(cuda_device):
    """The entry point's purpose: a render captured into a CUDA graph with no
    memory pool to draw on.  After one call outside the capture (the one-time
    symbol lookup), the call is captured on a side stream and replayed twice;
    each replay gives what an eager call gives."""
    lib = _lib.load()
    specs = [scenes.random_job(sh, seed=960 + sh, W=36 + 5 * sh, H=40, F=90) for sh in scenes.ALL_SHADERS]
    bufs = [scenes.initial_buffers(s) for s in specs]
    packed = pack(specs, [b[0] for b in bufs], [b[1] for b in bufs], cuda_device)
    b = packed.batch
    cfg = _lib.RastTiledConfig(16, 8, 0)
    assert lib.rast_tiled_workspace_bytes(ctypes.byref(b), ctypes.byref(cfg)) <= _lib.STATIC_SCRATCH_BYTES
    init = _snapshot(packed)
    stream = torch.cuda.current_stream(cuda_device)
    assert lib.rast_render_tiled_static(ctypes.byref(b), ctypes.byref(cfg), stream.cuda_stream) == 0
    torch.cuda.synchronize(cuda_device)
    expected = _snapshot(packed)
    _restore(packed, init)
    torch.cuda.synchronize(cuda_device)
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(cuda_device)
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            st = lib.rast_render_tiled_static(ctypes.byref(b), ctypes.byref(cfg), side.cuda_stream)
    assert st == 0
    torch.cuda.synchronize(cuda_device)
    for _ in range(2):
        _restore(packed, init)
        torch.cuda.synchronize(cuda_device)
        graph.replay()
        torch.cuda.synchronize(cuda_device)
        _assert_same(_snapshot(packed), expected)
    assert (expected[2] >= 0).any()


def test_static_scratch_rejects_batches_beyond_its_size(cuda_device):
    lib = _lib.load()
    spec = scenes.random_job(_lib.SHADER_DEPTH, seed=950)
    z0, _ = scenes.initial_buffers(spec)
    packed = pack([spec], [z0], [None], cuda_device)
    big = _lib.RastBatch.from_buffer_copy(packed.batch)
    big.total_setup = 4 << 20  # workspace far above the static array; checked before any launch
    cfg = _lib.RastTiledConfig(8, 8, 0)
    assert lib.rast_tiled_workspace_bytes(ctypes.byref(big), ctypes.byref(cfg)) > _lib.STATIC_SCRATCH_BYTES
    st = lib.rast_render_tiled_static(ctypes.byref(big), ctypes.byref(cfg), torch.cuda.current_stream(cuda_device).cuda_stream)
    assert st == 8
    assert lib.rast_error_string(st) == b"batch exceeds the static scratch of rast_render_tiled_static"


def test_static_scratch_refuses_tile_shapes_without_a_kernel(cuda_device):
    lib = _lib.load()
    spec = scenes.random_job(_lib.SHADER_DEPTH, seed=951)
    z0, _ = scenes.initial_buffers(spec)
    packed = pack([spec], [z0], [None], cuda_device)
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    for shape in ((0, 0), (0, 8), (5, 8)):
        cfg = _lib.RastTiledConfig(shape[0], shape[1], 0)
        assert lib.rast_render_tiled_static(ctypes.byref(packed.batch), ctypes.byref(cfg), stream) == 1
