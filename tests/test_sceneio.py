"""Scene files: the reference's OBJ/PLY import known-answer tests, the image readers on files
with known pixels, and the reference's own scene descriptions (copied into tests/golden/scenes by
tests/golden/make_scene_fixtures.py)."""
import math
import os
import struct
import zlib

import numpy as np
import pytest

from seesharp_gb300 import imagefile, sceneio
from seesharp_gb300.scene import InvalidOperationException, Matrix4x4

SCENES = os.path.join(os.path.dirname(__file__), "golden", "scenes")


# ---------------------------------------------------------------------------------------------
# SeeSharp.Tests/Core/Geometry/PlyFiles_Import.cs: a cube of six quads, ascii and binary
# ---------------------------------------------------------------------------------------------
_CUBE_V = [(0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0), (1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0)]
_CUBE_F = [(0, 1, 2, 3), (7, 6, 5, 4), (0, 4, 5, 1), (1, 5, 6, 2), (2, 6, 7, 3), (3, 7, 4, 0)]
_PLY_HEAD = ("ply\nformat {fmt} 1.0\ncomment a cube\nelement vertex 8\nproperty float x\nproperty float y\nproperty float z\n"
             "element face 6\nproperty list uchar int vertex_indices\nend_header\n")


@pytest.mark.parametrize("binary", [False, True])
def test_ply_cube_is_read_and_triangulated(tmp_path, binary):
    """PlyFiles_Import.cs:10-58: 12 triangles, 8 vertices, no material."""
    p = tmp_path / "test.ply"
    if binary:
        data = _PLY_HEAD.format(fmt="binary_little_endian").encode()
        data += b"".join(struct.pack("<3f", *v) for v in _CUBE_V)
        data += b"".join(struct.pack("<B4i", 4, *f) for f in _CUBE_F)
        p.write_bytes(data)
    else:
        body = "\n".join(" ".join(str(x) for x in v) for v in _CUBE_V) + "\n" + "\n".join("4 " + " ".join(map(str, f)) for f in _CUBE_F)
        p.write_text(_PLY_HEAD.format(fmt="ascii") + body)
    mesh = sceneio.read_ply(str(p))
    assert mesh.Material is None
    assert mesh.NumFaces == 12 and mesh.NumVertices == 8


# ---------------------------------------------------------------------------------------------
# SeeSharp.Tests/Core/Geometry/ObjFiles_Import.cs: a lone triangle, two quads in one group with
# two materials, and an emissive quad
# ---------------------------------------------------------------------------------------------
def _write_test_obj(d):
    obj = ["mtllib test.mtl", "v -1 0 -1", "v  1 0 -1", "v  0 1 -1", "g loner", "usemtl surface", "f 1 2 3",
           "v -1 -1 -2", "v  0 -1 -2", "v  0  1 -2", "v -1  1 -2", "v  0 -1 -2", "v  1 -1 -2", "v  1  1 -2", "v  0  1 -2",
           "g group", "usemtl surface", "f 4 5 6 7", "usemtl otherSurface", "f 8 9 10", "f 8 10 11"]
    for x, y in [(-0.1, -0.1), (0.1, -0.1), (0.1, 0.1), (-0.1, 0.1)]:
        obj += [f"v {x} {y} 2", "vn 0 0 -1"]
    obj += ["g light ", "usemtl light ", "f 12//1 13//2 14//3 15//4 "]
    (d / "test.obj").write_text("\n".join(obj) + "\n")
    (d / "test.mtl").write_text("\n newmtl surface\n Kd 0.9 0.7 0\n newmtl otherSurface\n Kd 0.1 0.1 0.9\n newmtl light\n Ke 10 10 10\n Kd 0 0 0\n")


def test_obj_is_read_with_materials_and_an_emitter(tmp_path):
    """ObjFiles_Import.cs:6-24."""
    _write_test_obj(tmp_path)
    f = sceneio.read_obj(str(tmp_path / "test.obj"))
    meshes, emitters = sceneio.obj_to_meshes(f, None)
    assert f.errors == []
    assert meshes and all(m.Material is not None for m in meshes)
    assert emitters


def test_obj_triangulation_and_one_mesh_per_material_group(tmp_path):
    """ObjFiles_Import.cs:26-51: 7 triangles in 4 meshes."""
    _write_test_obj(tmp_path)
    meshes, _ = sceneio.obj_to_meshes(sceneio.read_obj(str(tmp_path / "test.obj")), None)
    assert sum(m.NumFaces for m in meshes) == 7
    assert len(meshes) == 4


# ---------------------------------------------------------------------------------------------
# image readers on files with known pixels (encoded here from the format specifications)
# ---------------------------------------------------------------------------------------------
def _png_bytes(px, filters):
    h, w, ch = px.shape
    ctype = {1: 0, 3: 2, 4: 6}[ch]
    raw = b""
    prev = np.zeros(w * ch, np.int32)
    for y in range(h):
        line = px[y].reshape(-1).astype(np.int32)
        ft = filters[y % len(filters)]
        left = np.concatenate([np.zeros(ch, np.int32), line[:-ch]])
        upleft = np.concatenate([np.zeros(ch, np.int32), prev[:-ch]])
        if ft == 0:
            enc = line
        elif ft == 1:
            enc = line - left
        elif ft == 2:
            enc = line - prev
        elif ft == 3:
            enc = line - ((left + prev) >> 1)
        else:
            pa, pb, pc = np.abs(prev - upleft), np.abs(left - upleft), np.abs(left + prev - 2 * upleft)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
            enc = line - pred
        raw += bytes([ft]) + (enc & 0xFF).astype(np.uint8).tobytes()
        prev = line

    def chunk(t, body):
        return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)) + chunk(b"IDAT", zlib.compress(raw)) +
            chunk(b"IEND", b""))


@pytest.mark.parametrize("ch", [1, 3, 4])
def test_png_reader_decodes_every_filter(tmp_path, ch):
    rng = np.random.default_rng(ch)
    px = rng.integers(0, 256, size=(11, 7, ch), dtype=np.uint8)
    p = tmp_path / "t.png"
    p.write_bytes(_png_bytes(px, [0, 1, 2, 3, 4]))
    got = imagefile.read_png(str(p))
    want = imagefile.srgb_to_linear(px[..., :3] / 255.0) if ch >= 3 else imagefile.srgb_to_linear(np.repeat(px, 3, axis=2) / 255.0)
    assert got.shape == (11, 7, 3)
    assert np.allclose(got, want, atol=1e-7)


def _exr_bytes(rgb, compression, half):
    h, w, _ = rgb.shape
    ptype, dt = (1, np.float16) if half else (2, np.float32)

    def attr(name, typ, body):
        return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(body)) + body

    chl = b"".join(c.encode() + b"\0" + struct.pack("<iB3xii", ptype, 0, 1, 1) for c in "BGR") + b"\0"
    head = (struct.pack("<ii", 20000630, 2) + attr("channels", "chlist", chl) + attr("compression", "compression", bytes([compression])) +
            attr("dataWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1)) +
            attr("displayWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1)) + attr("lineOrder", "lineOrder", b"\0") +
            attr("pixelAspectRatio", "float", struct.pack("<f", 1)) + attr("screenWindowCenter", "v2f", struct.pack("<2f", 0, 0)) +
            attr("screenWindowWidth", "float", struct.pack("<f", 1)) + b"\0")
    lines = {0: 1, 3: 16}[compression]
    chunks = []
    for y0 in range(0, h, lines):
        n = min(lines, h - y0)
        blk = b"".join(rgb[y0 + r, :, c].astype(dt).astype(np.dtype(dt).newbyteorder("<")).tobytes() for r in range(n) for c in (2, 1, 0))
        if compression == 3:
            a = np.frombuffer(blk, np.uint8)
            re = np.concatenate([a[0::2], a[1::2]]).astype(np.int32)
            pred = re.copy()
            pred[1:] = (re[1:] - re[:-1] + 128 + 256) & 0xFF
            z = zlib.compress(pred.astype(np.uint8).tobytes())
            blk = z if len(z) < len(blk) else blk
        chunks.append(struct.pack("<ii", y0, len(blk)) + blk)
    table_len = 8 * len(chunks)
    offs, pos = [], len(head) + table_len
    for c in chunks:
        offs.append(pos)
        pos += len(c)
    return head + struct.pack(f"<{len(offs)}Q", *offs) + b"".join(chunks)


@pytest.mark.parametrize("compression,half", [(0, True), (0, False), (3, True), (3, False)])
def test_exr_reader_round_trip(tmp_path, compression, half):
    rng = np.random.default_rng(compression + half)
    rgb = rng.uniform(0, 50, size=(37, 23, 3)).astype(np.float32)
    if half:
        rgb = rgb.astype(np.float16).astype(np.float32)
    p = tmp_path / "t.exr"
    p.write_bytes(_exr_bytes(rgb, compression, half))
    assert np.array_equal(imagefile.read_exr(str(p)), rgb)


def test_reference_environment_map_decodes():
    """sunsky.exr (ZIP, FLOAT, 1600x900): a uniform sky with a small sun, finite and positive."""
    img = imagefile.read_exr(os.path.join(SCENES, "sunsky.exr"))
    assert img.shape == (900, 1600, 3) and np.isfinite(img).all() and img.min() >= 0
    sun = img[..., 0] > 10
    assert 0 < sun.sum() < 1000 and img.max() > 100
    assert np.allclose(img[0, 0], img[899, 1599]) and np.allclose(img[0, 0], [0.4232657, 0.70456624, 0.8605181])


# ---------------------------------------------------------------------------------------------
# transforms (IO/JsonScene.cs:144-183) and the reference's scene files
# ---------------------------------------------------------------------------------------------
def test_yaw_pitch_roll_matches_single_axis_rotations():
    a = 0.7
    c, s = math.cos(a), math.sin(a)
    rx = np.array([[1, 0, 0, 0], [0, c, s, 0], [0, -s, c, 0], [0, 0, 0, 1]], np.float32)
    rz = np.array([[c, s, 0, 0], [-s, c, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], np.float32)
    assert np.allclose(Matrix4x4.CreateFromYawPitchRoll(0, a, 0), rx, atol=1e-6)
    assert np.allclose(Matrix4x4.CreateFromYawPitchRoll(a, 0, 0), Matrix4x4.CreateRotationY(a), atol=1e-6)
    assert np.allclose(Matrix4x4.CreateFromYawPitchRoll(0, 0, a), rz, atol=1e-6)


@pytest.mark.parametrize("name,meshes,tris,emitters,background", [
    ("CornellBox/CornellBox.json", 8, 36, 2, False), ("simpledi.json", 2, 4, 2, False), ("simplebackground.json", 1, 2, 0, True),
    ("furnacebox.json", 1, 12, 0, False), ("TextureTest/TextureTest.json", 3, 6, 2, False), ("ExampleScene/ExampleScene.json", 10, 21840, 20, False)])
def test_reference_scene_files_load(name, meshes, tris, emitters, background):
    sc = sceneio.load_json_scene(os.path.join(SCENES, name))
    assert len(sc.Meshes) == meshes and sum(m.NumFaces for m in sc.Meshes) == tris
    assert len(sc.Emitters) == emitters and (sc.Background is not None) == background
    assert all(m.Material is not None for m in sc.Meshes)


def test_cornell_box_camera_and_materials():
    sc = sceneio.load_json_scene(os.path.join(SCENES, "CornellBox", "CornellBox.json"))
    w2c = sc.Camera.WorldToCamera
    assert np.allclose(w2c[3, :3], [0, -1, -6.8], atol=1e-6) and np.allclose(w2c[:3, :3], np.eye(3))
    assert sc.Camera.VerticalFieldOfView == pytest.approx(19.5)
    left = [m for m in sc.Meshes if m.Material.Name == "LeftWall"][0]
    assert np.allclose(left.Material.MaterialParameters.BaseColor.constColor.array(), [0.63, 0.065, 0.05])


def test_camera_rotation_looks_down_in_simpledi():
    """rotation (-90, 0, 0): pitch -90 degrees, so the camera's -z axis points down (-y)."""
    sc = sceneio.load_json_scene(os.path.join(SCENES, "simpledi.json"))
    ok, c2w = Matrix4x4.Invert(sc.Camera.WorldToCamera)
    fwd = np.array([0, 0, -1, 0], np.float32) @ c2w
    assert np.allclose(fwd[:3], [0, -1, 0], atol=1e-6)
    assert np.allclose(c2w[3, :3], [0, 1, 0], atol=1e-6)


def test_scene_without_lights_is_rejected_like_the_reference():
    sc = sceneio.load_json_scene(os.path.join(SCENES, "furnacebox.json"))
    from seesharp_gb300 import FrameBuffer
    sc.FrameBuffer = FrameBuffer(8, 8)
    with pytest.raises(InvalidOperationException):
        sc.Prepare()
