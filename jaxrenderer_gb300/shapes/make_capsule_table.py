"""Regenerate capsule_table.npz from the reference's tabulated capsule
sphere (renderer/shapes/capsule.py:19-1956 of JoeyTeng/jaxrenderer v0.3.2,
the textured sphere of tinyrenderer's create_capsule that it cites).

The table's literals are read with `ast` (the reference module imports JAX,
so it is not imported) and stored as the float32 / int32 arrays
jnp.array makes of them: 576 vertices, 576 normals, 576 uvs, 192 faces.

    python -m jaxrenderer_gb300.shapes.make_capsule_table [REFERENCE_ROOT]
"""
import ast
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
NAMES = {"_verts": ("verts", np.float32), "_normals": ("normals", np.float32), "_uvs": ("uvs", np.float32),
         "_faces": ("faces", np.int32)}


def main(reference_root: str = "/root/reference") -> None:
    src = Path(reference_root) / "renderer" / "shapes" / "capsule.py"
    tree = ast.parse(src.read_text())
    out = {}
    for node in ast.walk(tree):
        if isinstance(node, (ast.AnnAssign, ast.Assign)):
            target = node.target if isinstance(node, ast.AnnAssign) else node.targets[0]
            if isinstance(target, ast.Name) and target.id in NAMES and isinstance(node.value, ast.Call):
                name, dtype = NAMES[target.id]
                out[name] = np.asarray(ast.literal_eval(node.value.args[0]), dtype=dtype)
    assert set(out) == {n for n, _ in NAMES.values()}, sorted(out)
    np.savez_compressed(HERE / "capsule_table.npz", **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main(*sys.argv[1:])
