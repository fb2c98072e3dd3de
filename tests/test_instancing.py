"""Instanced scenes on the host: instance-table offsets, the reference
host path (merge_objects + flatten_corners) the device merge is checked
against, and the sequential global norm both sides use."""
import numpy as np

from jaxrenderer_gb300 import synthetic
from jaxrenderer_gb300.geometry import normalise


def test_instance_table_offsets():
    inst = synthetic.brax_like_instances(5, seed=synthetic.BASE_SEED + 31)
    t = inst.instance_table()
    lib = inst.library.table
    corner = 0
    for s in range(inst.n_scenes):
        a, b = int(inst.scene_begin[s]), int(inst.scene_begin[s + 1])
        offs = {"vert_offset": 0, "norm_offset": 0, "uv_offset": 0}
        for i in range(a, b):
            m = lib[inst.mesh[i]]
            assert t["scene_first"][i] == a and t["scene_count"][i] == b - a
            for k, field in (("vert_offset", "n_verts"), ("norm_offset", "n_norms"), ("uv_offset", "n_uvs")):
                assert t[k][i] == offs[k]
                offs[k] += int(m[field])
            assert t["corner_begin"][i] == corner
            corner += 3 * int(m["n_faces"])
        for i in range(a, b):
            assert t["scene_verts"][i] == offs["vert_offset"]
            assert t["scene_uvs"][i] == offs["uv_offset"]
    assert inst.corner_begin()[-1] + 3 * inst.n_faces[-1] == corner


def test_host_flat_matches_per_scene_merge():
    inst = synthetic.brax_like_instances(3, seed=synthetic.BASE_SEED + 32)
    flat = inst.host_flat([0, 1, 2])
    one = inst.host_flat([1])
    rows = slice(int(flat.corner_begin[1]), int(flat.corner_begin[1] + 3 * flat.n_faces[1]))
    np.testing.assert_array_equal(flat.position[rows], one.position)
    np.testing.assert_array_equal(flat.texture_index[rows], one.texture_index)
    assert flat.n_faces.tolist() == inst.n_faces.tolist()
    # ground first: its two faces sample object 0's map
    assert (flat.texture_index[:6] == 0).all()
    # object normals come out scaled by one global norm per object (unit-free)
    assert np.isfinite(flat.normal).all()


def test_global_norm_is_sequential():
    v = np.random.default_rng(0).normal(size=(1000, 3)).astype(np.float32)
    acc = np.float32(0)
    for x in v.reshape(-1):
        acc = np.float32(acc + np.float32(x * x))
    np.testing.assert_array_equal(normalise(v), v / np.sqrt(acc))
