"""Copies the reference's loadable example scenes into this folder.

Radiantium ships no tests and no numeric fixtures; its example scene files
(Example/**.json) and the OBJ meshes they load are the only inputs of its
own that pin the JSON -> RendererBuilder.Build -> flattened scene path.  This
script copies, byte for byte, every example scene whose assets are present in
the reference's tree and which uses only plugins on the GPU path, keeping the
reference's layout (a scene's "../assets/..." locations resolve unchanged),
and records a SHA-256 of each file in MANIFEST.sha256.  Scenes that need
assets the reference does not ship (bunny.obj, ajax.obj, the .exr maps) or
plugins off the path (bdpt, subsurface, disney) are left out.

    python tests/fixtures/reference/copy_reference_scenes.py [reference root]
"""
import hashlib
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

SCENES = [
    "cbox/mis_test.json", "cbox/vol_test.json", "cbox/vol_test2.json", "cbox/teapot.json",
    "cbox/anis_rough_metal.json", "cbox/anis_rough_glass.json", "cbox/anis_rough_plastic.json",
    "cbox/test_rough_glass.json", "cbox/test_adjoint_particle.json",
    "veach_mi/mis.json", "veach_mi/nee.json", "veach_mi/bxdf.json", "veach_mi/particle.json",
    "veach_bidir/path.json", "veach_bidir/particle.json",
]
ASSETS = ["assets/cbox/walls.obj", "assets/cbox/leftwall.obj", "assets/cbox/rightwall.obj", "assets/cbox/light.obj",
          "assets/teapot.obj", "assets/rect.obj"] + \
         [f"assets/veach_mi/{n}.obj" for n in ("floor", "plate1", "plate2", "plate3", "plate4")] + \
         [f"assets/veach_bidir/Mesh{i:03d}.obj" for i in range(12)]


def main(ref_root):
    example = os.path.join(ref_root, "Example")
    lines = []
    for rel in SCENES + ASSETS:
        dst = os.path.join(HERE, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(os.path.join(example, rel), dst)
        with open(dst, "rb") as f:
            lines.append(f"{hashlib.sha256(f.read()).hexdigest()}  {rel}\n")
    with open(os.path.join(HERE, "MANIFEST.sha256"), "w") as f:
        f.writelines(lines)
    print(f"copied {len(SCENES)} scenes and {len(ASSETS)} assets from {example}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
