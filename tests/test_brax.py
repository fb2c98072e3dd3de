"""Batched Brax inputs on the host: the reference-format pickle loader (no
JAX; only whitelisted reconstructors), frames -> instanced scenes, and the
structure of the reference's own fixture where it is available."""
import os
import pickle
from pathlib import Path

import numpy as np
import pytest

from jaxrenderer_gb300 import brax, synthetic
from jaxrenderer_gb300.model import Model, ModelObject
from jaxrenderer_gb300.renderer import CameraParameters
from tests.brax_format import reference_pickle

REFERENCE = Path(os.environ.get("JAXRENDERER_REFERENCE", "/root/reference"))


def test_reference_format_round_trip():
    objects, camera, target = synthetic.ant_like_batched(3)
    got_objects, got_camera, got_target = brax.load_batched_inputs(reference_pickle(objects, camera, target))
    assert len(got_objects) == 18 and isinstance(got_objects[0], ModelObject)
    assert isinstance(got_objects[0].model, Model) and isinstance(got_camera, CameraParameters)
    for a, b in zip(objects, got_objects):
        np.testing.assert_array_equal(a.transform, b.transform)
        np.testing.assert_array_equal(a.model.verts, b.model.verts)
        np.testing.assert_array_equal(a.model.diffuse_map, b.model.diffuse_map)
    np.testing.assert_array_equal(camera.position, got_camera.position)
    np.testing.assert_array_equal(target, got_target)


def test_loader_refuses_other_globals():
    with pytest.raises(pickle.UnpicklingError):
        brax.load_batched_inputs(pickle.dumps(os.getcwd))


def test_frames_become_instanced_scenes():
    objects, camera, target = synthetic.ant_like_batched(3)
    bb = brax.scenes_from_batched(objects, camera, target, repeat=2)
    inst = bb.scenes
    assert inst.n_scenes == 6 and inst.n_faces.tolist() == [3276] * 6
    assert inst.library.table.shape[0] == 18  # ground + 17 distinct capsules
    for s, f in ((0, 0), (4, 1)):
        for got, o in zip(inst.objects(s), objects):
            np.testing.assert_array_equal(got.transform, o.transform[f])
            np.testing.assert_array_equal(got.model.diffuse_map, o.model.diffuse_map[f])
            np.testing.assert_array_equal(got.model.faces, o.model.faces[f])
    assert bb.camera.viewWidth == 960 and bb.camera.viewHeight == 540
    np.testing.assert_array_equal(bb.shadow.centre[4], target[1])


@pytest.mark.skipif(not (REFERENCE / "test_resources/pre-gen-brax/inputs-2.zip").exists(),
                    reason="the reference's fixtures are not on this machine")
def test_reference_fixture_structure():
    objects, camera, target = brax.load_batched_inputs(str(REFERENCE / "test_resources/pre-gen-brax/inputs-2.zip"))
    bb = brax.scenes_from_batched(objects, camera, target)
    assert bb.scenes.n_scenes == 2 and len(objects) == 18
    assert bb.scenes.n_faces.tolist() == [3276, 3276]
    assert (bb.camera.viewWidth, bb.camera.viewHeight) == (960, 540)


GOLDEN = Path(__file__).resolve().parent / "golden"


def test_npz_archive_round_trip(tmp_path):
    objects, camera, target = synthetic.ant_like_batched(3)
    path = tmp_path / "ant.npz"
    brax.save_batched_npz(path, objects, camera, target)
    got_objects, got_camera, got_target = brax.load_batched_npz(path)
    for a, b in zip(objects, got_objects):
        for field in ("local_scaling", "transform", "double_sided"):
            np.testing.assert_array_equal(np.asarray(getattr(a, field)), np.asarray(getattr(b, field)))
        for field in a.model._fields:
            np.testing.assert_array_equal(np.asarray(getattr(a.model, field)), np.asarray(getattr(b.model, field)))
    for field in camera._fields:
        np.testing.assert_array_equal(np.asarray(getattr(camera, field)), np.asarray(getattr(got_camera, field)))
    np.testing.assert_array_equal(target, got_target)


def test_committed_fixture_archives():
    """tests/golden/brax_ant_{2,30}.npz: the reference's inputs-{2,30}.zip
    (SHA-256 recorded in each archive), 18 objects, 3,276 triangles per frame."""
    for n, sha in ((2, "38d050833a0307409f28b5ed2633a7b8f3e14287cf607a4df9426872e8192db3"),
                   (30, "0ef2738b6c4cee12b94b2569679ff71598b27df77dc53dd9762302f9d71fab7f")):
        with np.load(GOLDEN / f"brax_ant_{n}.npz") as z:
            assert str(z["source_sha256"]) == sha
        objects, camera, target = brax.load_batched_npz(GOLDEN / f"brax_ant_{n}.npz")
        bb = brax.scenes_from_batched(objects, camera, target)
        assert bb.scenes.n_scenes == n and bb.scenes.n_faces.tolist() == [3276] * n
        assert (bb.camera.viewWidth, bb.camera.viewHeight) == (960, 540)


@pytest.mark.skipif(not (REFERENCE / "test_resources/pre-gen-brax/inputs-30.zip").exists(),
                    reason="the reference's fixtures are not on this machine")
@pytest.mark.parametrize("n", [2, 30])
def test_fixture_archives_equal_the_reference_pickles(n):
    import hashlib

    src = REFERENCE / f"test_resources/pre-gen-brax/inputs-{n}.zip"
    with np.load(GOLDEN / f"brax_ant_{n}.npz") as z:
        assert str(z["source_sha256"]) == hashlib.sha256(src.read_bytes()).hexdigest()
    ref = brax.load_batched_inputs(str(src))
    got = brax.load_batched_npz(GOLDEN / f"brax_ant_{n}.npz")
    for a, b in zip(ref[0], got[0]):
        for field in ("local_scaling", "transform", "double_sided"):
            np.testing.assert_array_equal(np.asarray(getattr(a, field)), np.asarray(getattr(b, field)))
        for field in a.model._fields:
            np.testing.assert_array_equal(np.asarray(getattr(a.model, field)), np.asarray(getattr(b.model, field)))
    for field in ref[1]._fields:
        np.testing.assert_array_equal(np.asarray(getattr(ref[1], field)), np.asarray(getattr(got[1], field)))
    np.testing.assert_array_equal(ref[2], got[2])
