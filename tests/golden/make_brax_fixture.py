"""Regenerate tests/golden/brax_ant_{2,30}.npz from the reference's Brax Ant
inputs (test_resources/pre-gen-brax/inputs-{2,30}.zip of
JoeyTeng/jaxrenderer v0.3.2: pickles of batched ModelObjects, batched
CameraParameters and the per-frame camera target, 960x540, 2 and 30 frames).

The pickles are read without JAX by jaxrenderer_gb300.brax's whitelisting
unpickler and re-written as pickle-free .npz archives (save_batched_npz);
each archive records the SHA-256 of the zip it came from.

    python tests/golden/make_brax_fixture.py [REFERENCE_ROOT]
"""
import hashlib
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from jaxrenderer_gb300 import brax  # noqa: E402


def main(reference_root: str = "/root/reference") -> None:
    src_dir = Path(reference_root) / "test_resources" / "pre-gen-brax"
    for n in (2, 30):
        src = src_dir / f"inputs-{n}.zip"
        sha = hashlib.sha256(src.read_bytes()).hexdigest()
        objects, camera, target = brax.load_batched_inputs(str(src))
        out = HERE / f"brax_ant_{n}.npz"
        brax.save_batched_npz(out, objects, camera, target, source_sha256=sha)
        print(out.name, out.stat().st_size, "bytes from", src.name, sha)


if __name__ == "__main__":
    main(*sys.argv[1:])
