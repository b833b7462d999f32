"""Copies the reference's own scene files (SeeSharp Data/Scenes and the template's ExampleScene)
into tests/golden/scenes/, unchanged, so that the scene-loading tests and the GPU parity tests
of those scenes run without the reference checkout.

Usage: python tests/golden/make_scene_fixtures.py /path/to/SeeSharp
"""
import os
import shutil
import sys

FILES = [
    "Data/Scenes/CornellBox/CornellBox.json",
    "Data/Scenes/CornellBox/References/Config.json",
    "Data/Scenes/CornellBox/References/MaxDepth5-Width512-Height512.json",
    "Data/Scenes/CornellBox/References/MaxDepth2-Width512-Height512.json",
    "Data/Scenes/simpledi.json",
    "Data/Scenes/simplebackground.json",
    "Data/Scenes/sunsky.exr",
    "Data/Scenes/furnacebox.json",
    "Data/Scenes/TextureTest/TextureTest.json",
    "Data/Scenes/TextureTest/TextureTest.obj",
    "Data/Scenes/TextureTest/Textures/TestPattern.png",
    "SeeSharp.Templates/content/SeeSharp.Template/Scenes/ExampleScene/ExampleScene.json",
]
PLY_DIR = "SeeSharp.Templates/content/SeeSharp.Template/Scenes/ExampleScene/Meshes"


def main(src):
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "scenes")
    files = list(FILES) + [os.path.join(PLY_DIR, f) for f in sorted(os.listdir(os.path.join(src, PLY_DIR))) if f.endswith(".ply")]
    for rel in files:
        dst_rel = rel.replace("Data/Scenes/", "").replace("SeeSharp.Templates/content/SeeSharp.Template/Scenes/", "")
        dst = os.path.join(out, dst_rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(os.path.join(src, rel), dst)
        print(dst_rel, os.path.getsize(dst))


if __name__ == "__main__":
    main(sys.argv[1])
