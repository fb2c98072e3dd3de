"""The compiled primitive_chooser / mix hooks (layered chooser, nearest and
"over" mixers) on the CPU: the oracle's restatement is pinned against a
Python transcription of the hook semantics built from single-face renders,
and the host side (hook objects, job validation) is checked.  No GPU."""
import copy

import numpy as np
import pytest

from jaxrenderer_gb300 import _lib, hooks
from jaxrenderer_gb300.shader import Shader
from jaxrenderer_gb300.shaders import GouraudShader, PhongReflectionTextureShader
from oracle import oracle
from tests import scenes

F32 = np.float32


def _single_face(spec, p, shader=None):
    s = copy.copy(spec)
    s.faces = spec.faces[p : p + 1]
    s.layers, s.mixer, s.face_alpha = 1, _lib.MIX_NEAREST, None
    if shader is not None:
        s.shader = shader
    return s


def per_face_fragments(spec):
    """For every face p, rendered alone: where it is a chooser candidate
    (keep & inside & front, depth not +inf) with its depth, and where its
    fragment shader keeps it, with its colour."""
    W, H = spec.width, spec.height
    z0 = np.full((W, H), np.inf, F32)
    c0 = np.zeros((W, H, 3), F32)
    out = []
    for p in range(spec.n_faces):
        geo = oracle.render(_single_face(spec, p, _lib.SHADER_DEPTH), z0)
        frag = oracle.render(_single_face(spec, p), z0, c0)
        out.append((geo["prim_id"] == 0, geo["zbuffer"], frag["prim_id"] == 0, frag["canvas"]))
    return out


def _order(z, p):
    """The chooser's order: NaN first, -0 == +0, then ascending; index on ties."""
    return (0, 0.0, p) if np.isnan(z) else (1, float(z), p)


def transcribe(spec, frags, z0, c0):
    """The hook semantics written out per pixel in float32 scalar arithmetic."""
    W, H = spec.width, spec.height
    z, c = z0.copy(), c0.copy()
    pid = np.full((W, H), -1, np.int32)
    alpha = None if spec.face_alpha is None else np.asarray(spec.face_alpha, F32)
    bg = np.broadcast_to(np.asarray(spec.background, F32), (3,))
    one = F32(1.0)
    for i in range(W):
        for j in range(H):
            cands = [(frags[p][1][i, j], p) for p in range(len(frags)) if frags[p][0][i, j]]
            slots = sorted(cands, key=lambda t: _order(*t))[: spec.layers]
            kept = [(zz, p) for zz, p in slots if frags[p][2][i, j]]
            if not kept:
                continue
            z[i, j] = kept[0][0]
            pid[i, j] = kept[0][1]
            if spec.mixer == _lib.MIX_NEAREST:
                c[i, j] = frags[kept[0][1]][3][i, j]
                continue
            T, C = one, np.zeros(3, F32)
            for _, p in kept:
                a = alpha[p] if alpha is not None else F32(spec.opacity)
                w = F32(T * a)
                for k in range(3):
                    C[k] = F32(C[k] + F32(w * frags[p][3][i, j, k]))
                T = F32(T * F32(one - a))
            for k in range(3):
                c[i, j, k] = F32(C[k] + F32(T * bg[k]))
    return z, c, pid


CASES = [
    (_lib.SHADER_PHONG_REFLECTION, 1, _lib.MIX_NEAREST, None),
    (_lib.SHADER_PHONG_REFLECTION, 3, _lib.MIX_OVER, 0.4),
    (_lib.SHADER_PHONG_REFLECTION, 4, _lib.MIX_OVER, "per_face"),
    (_lib.SHADER_GOURAUD, 2, _lib.MIX_NEAREST, None),
    (_lib.SHADER_GOURAUD, 4, _lib.MIX_OVER, "per_face"),
]


@pytest.mark.parametrize("shader,layers,mixer,opacity", CASES)
def test_oracle_layers_match_transcription(shader, layers, mixer, opacity):
    spec = scenes.random_job(shader, seed=40 + layers, W=20, H=16, F=36, spread=0.9)
    spec.layers, spec.mixer = layers, mixer
    rng = np.random.Generator(np.random.PCG64(7 + layers))
    if opacity == "per_face":
        spec.face_alpha = rng.uniform(0.1, 0.9, spec.n_faces).astype(F32)
    elif opacity is not None:
        spec.opacity = opacity
    spec.background = (0.25, 0.5, 0.75)
    z0, c0 = scenes.initial_buffers(spec)
    frags = per_face_fragments(spec)
    want_z, want_c, want_p = transcribe(spec, frags, z0, c0)
    got = oracle.render(spec, z0, c0)
    np.testing.assert_array_equal(got["prim_id"], want_p)
    np.testing.assert_array_equal(got["zbuffer"].view(np.uint32), want_z.view(np.uint32))
    np.testing.assert_array_equal(got["canvas"].view(np.uint32), want_c.view(np.uint32))
    # several layers actually overlap somewhere
    depth_hits = sum(f[0].astype(np.int32) for f in frags)
    assert depth_hits.max() >= 2
    if shader == _lib.SHADER_GOURAUD:  # the fragment shader discards some candidates
        assert any((f[0] & ~f[2]).any() for f in frags)


def test_oracle_one_layer_is_the_default_chooser_where_it_finds_a_candidate():
    spec = scenes.random_job(_lib.SHADER_PHONG_REFLECTION, seed=5, F=60)
    z0, c0 = scenes.initial_buffers(spec)
    default = oracle.render(spec, z0, c0)
    spec.layers = 1
    layered = oracle.render(spec, z0, c0)
    found = layered["prim_id"] >= 0
    assert found.any()
    np.testing.assert_array_equal(layered["prim_id"][found], default["prim_id"][found])
    np.testing.assert_array_equal(layered["canvas"][found], default["canvas"][found])
    # elsewhere the default chooser may still write its fallback, primitive 0
    assert set(np.unique(default["prim_id"][~found])) <= {-1, 0}


# ------------------------------------------------------------------- host side


class Glass(PhongReflectionTextureShader):
    primitive_chooser = hooks.LayeredChooser(3)
    mix = hooks.OverMixer(opacity=0.5, background=(1.0, 1.0, 1.0))


class PeelGouraud(GouraudShader):
    primitive_chooser = hooks.LayeredChooser(2)


def test_hooks_of_builtin_and_hooked_shaders():
    assert hooks.hooks_of(PhongReflectionTextureShader, 10)["layers"] == 0
    h = hooks.hooks_of(Glass, 10)
    assert (h["layers"], h["mixer"], h["opacity"], h["background"]) == (3, _lib.MIX_OVER, 0.5, (1.0, 1.0, 1.0))
    h = hooks.hooks_of(PeelGouraud, 10)
    assert (h["layers"], h["mixer"]) == (2, _lib.MIX_NEAREST)

    class PerFace(PhongReflectionTextureShader):
        primitive_chooser = hooks.LayeredChooser(2)
        mix = hooks.OverMixer(opacity=np.linspace(0, 1, 4))

    assert hooks.hooks_of(PerFace, 4)["face_alpha"].shape == (4,)
    with pytest.raises(ValueError):
        hooks.hooks_of(PerFace, 5)


def test_python_overrides_are_refused():
    class PyChooser(PhongReflectionTextureShader):
        @staticmethod
        def primitive_chooser(*args):
            return args

    class PyMix(PhongReflectionTextureShader):
        @staticmethod
        def mix(*args):
            return args

    class OverOnly(PhongReflectionTextureShader):
        mix = hooks.OverMixer(0.5)

    with pytest.raises(NotImplementedError):
        hooks.hooks_of(PyChooser, 1)
    with pytest.raises(NotImplementedError):
        hooks.hooks_of(PyMix, 1)
    with pytest.raises(ValueError):
        hooks.hooks_of(OverOnly, 1)
    with pytest.raises(ValueError):
        hooks.LayeredChooser(_lib.MAX_LAYERS + 1)
    assert Shader.primitive_chooser is PhongReflectionTextureShader.primitive_chooser


@pytest.mark.parametrize("field,value", [("layers", -1), ("layers", _lib.MAX_LAYERS + 1), ("mixer", 2),
                                         ("depth_layers", 1), ("over_without_layers", 0)])
def test_validate_job_rejects_bad_hooks(field, value):
    lib = _lib.load()
    spec = scenes.random_job(_lib.SHADER_PHONG_REFLECTION, seed=1, F=4)
    J = _lib.RastJob()
    J.shader, J.width, J.height, J.n_verts, J.n_faces = spec.shader, 8, 8, spec.n_verts, spec.n_faces
    J.tex_w = J.tex_h = J.tex_c = 3
    J.n_objects, J.spec_w, J.spec_h = 1, 2, 2
    assert lib.rast_validate_job(J) == 0
    J.layers, J.mixer = 2, _lib.MIX_OVER
    assert lib.rast_validate_job(J) == 0
    if field == "depth_layers":
        J.shader = _lib.SHADER_DEPTH
    elif field == "over_without_layers":
        J.layers = 0
    else:
        setattr(J, field, value)
    assert lib.rast_validate_job(J) == 1  # RAST_ERR_INVALID_ARGUMENT
