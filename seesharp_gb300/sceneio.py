"""Scene files: SeeSharp's .json scene description with inline triangle meshes, Wavefront .obj
(+ .mtl) and .ply meshes, feeding the same Scene objects that Scene.Prepare uploads with sst_scene_*.

Follows the reference loaders:

* `load_json_scene`  -> JsonScene.LoadFromFile (IO/JsonScene.cs:189-216): named transforms
  (:144-183), cameras (:128-142), background (:114-126), materials (:53-112), objects (:17-51),
  exposure; JsonUtils (IO/JsonUtils.cs) for colours, textures and matrices.
* `TriMeshLoader`    -> IO/TriMeshLoader.cs:8-64 (type "trimesh").
* `read_obj` + `obj_to_meshes` -> ObjMesh.FromFile / ParseObjFile / ParseMtlFile
  (IO/ObjMesh.cs:178-479) and ObjConverter.CreateMeshes (IO/ObjConverter.cs:31-215) (type "obj").
* `read_ply`         -> PlyFile.ParseFile / ToMesh (IO/PlyFile.cs:42-410) (type "ply").

Images referenced by the scene (textures, the environment map) are read by `imagefile`.
"""
from __future__ import annotations

import json
import math
import os
import re
import struct

import numpy as np

from .images import MonochromeImage, RgbColor, RgbImage, TextureMono, TextureRgb
from .imagefile import read_image
from .scene import (DiffuseEmitter, DiffuseMaterial, EnvironmentMap, GenericMaterial, GlossyEmitter, Matrix4x4, Mesh, PerspectiveCamera,
                    Scene)


class MeshLoadException(RuntimeError):
    """IO/MeshLoadException.cs: a corrupt or unsupported mesh file."""


# ---------------------------------------------------------------------------------------------
# JsonUtils (IO/JsonUtils.cs)
# ---------------------------------------------------------------------------------------------
def _vec3(v):
    return np.array([float(v[0]), float(v[1]), float(v[2])], np.float32)


def _rgb(elem):
    v = _vec3(elem["value"])
    return RgbColor(*v)


def _texture_rgb(elem, scene_path, cache):
    typ = elem["type"]
    if typ == "rgb":
        return TextureRgb(_rgb(elem))
    if typ == "image":
        return TextureRgb(_load_rgb_image(os.path.join(os.path.dirname(scene_path), elem["filename"]), cache))
    return TextureRgb(RgbColor(1, 0, 1))   # invalid specification: magenta (JsonUtils.cs:24-27)


def _float_or_texture(mat, name, scene_path, default, cache):
    if name not in mat:
        return TextureMono(default)
    v = mat[name]
    if isinstance(v, (int, float)):
        return TextureMono(float(v))
    img = _load_rgb_image(os.path.join(os.path.dirname(scene_path), v), cache)
    # a monochrome image from an RGB file: the channel mean
    return TextureMono(MonochromeImage(img.data.mean(axis=2, keepdims=True)))


def _matrix(arr):
    """JsonUtils.GetMatrix (IO/JsonUtils.cs:51-88): 12 or 16 row-major entries."""
    n = len(arr)
    if n not in (9, 12, 16):
        return Matrix4x4.Identity()
    if n == 9:
        # the reference reads entry 10 for M33, which a 9-entry array does not have
        raise IndexError("a 9-entry matrix reads past its end (JsonUtils.GetMatrix)")
    a = [float(x) for x in arr]
    m = np.eye(4, dtype=np.float32)
    m[0, 0:3] = a[0:3]
    m[1, 0:3] = a[4:7]
    m[2, 0:3] = a[8:11]
    m[0, 3], m[1, 3], m[2, 3] = a[3], a[7], a[11]
    if n == 16:
        m[3, :] = a[12:16]
    return m


def _optional(d, name, default):
    return d[name] if name in d else default


def _load_rgb_image(path, cache):
    key = os.path.abspath(path)
    if key not in cache:
        cache[key] = RgbImage(read_image(path))
    return cache[key]


# ---------------------------------------------------------------------------------------------
# transforms, cameras, background, materials (IO/JsonScene.cs)
# ---------------------------------------------------------------------------------------------
def _named_transforms(root):
    out = {}
    for t in root["transforms"]:
        m = Matrix4x4.Identity()
        if "scale" in t:
            s = _vec3(t["scale"])
            m = m @ Matrix4x4.CreateScale(*s)
        if "rotation" in t:
            r = _vec3(t["rotation"]).astype(np.float64) * (math.pi / 180.0)
            m = m @ Matrix4x4.CreateFromYawPitchRoll(float(np.float32(r[1])), float(np.float32(r[0])), float(np.float32(r[2])))
        if "position" in t:
            p = _vec3(t["position"])
            m = m @ Matrix4x4.CreateTranslation(*p)
        if "matrix" in t:
            m = _matrix(t["matrix"])
        out[t["name"]] = m.astype(np.float32)
    return out


def _cameras(scene, root, transforms):
    for c in root["cameras"]:
        ok, w2c = Matrix4x4.Invert(transforms[c["transform"]])
        scene.Camera = PerspectiveCamera(w2c, float(c["fov"]))


def _materials(scene_path, root, cache):
    named, emissive = {}, {}
    for m in root.get("materials", []):
        name = m["name"]
        typ = m.get("type", "generic")
        if typ == "diffuse":
            p = DiffuseMaterial.Parameters(BaseColor=_texture_rgb(m["baseColor"], scene_path, cache), Transmitter=bool(_optional(m, "thin", False)))
            named[name] = DiffuseMaterial(p)
        else:
            p = GenericMaterial.Parameters(
                BaseColor=_texture_rgb(m["baseColor"], scene_path, cache),
                Roughness=_float_or_texture(m, "roughness", scene_path, 0.5, cache),
                Anisotropic=float(_optional(m, "anisotropic", 0.0)),
                IndexOfRefraction=float(_optional(m, "IOR", 1.01)),
                Metallic=float(_optional(m, "metallic", 0.0)),
                SpecularTintStrength=float(_optional(m, "specularTint", 0.0)),
                SpecularTransmittance=float(_optional(m, "specularTransmittance", 0.0)))
            named[name] = GenericMaterial(p)
        named[name].Name = name
        if "emission" in m:
            e = _rgb(m["emission"])
            if np.any(e.array() != 0):
                emissive[name] = (e, bool(_optional(m, "emissionIsGlossy", False)), float(_optional(m, "emissionExponent", 50.0)))
    return named, emissive


def _emitters_for(mesh, material_name, emissive, obj):
    if material_name in emissive:
        rad, glossy, exponent = emissive[material_name]
        return GlossyEmitter.MakeFromMesh(mesh, rad, exponent) if glossy else DiffuseEmitter.MakeFromMesh(mesh, rad)
    if obj is not None and "emission" in obj:
        return DiffuseEmitter.MakeFromMesh(mesh, _rgb(obj["emission"]))
    return []


# ---------------------------------------------------------------------------------------------
# mesh loaders
# ---------------------------------------------------------------------------------------------
def _load_trimesh(obj, named, emissive, dirname):
    """TriMeshLoader.LoadMesh (IO/TriMeshLoader.cs:8-64)."""
    mat_name = obj["material"]
    material = named[mat_name]
    V = np.asarray(obj["vertices"], np.float32).reshape(-1, 3)
    I = np.asarray(obj["indices"], np.int32)
    N = np.asarray(obj["normals"], np.float32).reshape(-1, 3) if "normals" in obj else None
    UV = np.asarray(obj["uv"], np.float32).reshape(-1, 2) if "uv" in obj else None
    mesh = Mesh(V, I, shadingNormals=N, textureCoordinates=UV)
    mesh.Material = material
    return [mesh], _emitters_for(mesh, mat_name, emissive, obj)


def _load_ply_object(obj, named, emissive, dirname):
    """PlyLoader.LoadMesh (IO/PlyLoader.cs:11-39)."""
    mat_name = obj["material"]
    material = named[mat_name]
    mesh = read_ply(os.path.join(dirname, obj["relativePath"]))
    mesh.Material = material
    return [mesh], _emitters_for(mesh, mat_name, emissive, obj)


def _load_obj_object(obj, named, emissive, dirname):
    """ObjConverter.LoadMesh (IO/ObjConverter.cs:217-228): the .json materials replace
    equally named .mtl materials."""
    parsed = read_obj(os.path.join(dirname, obj["relativePath"]))
    return obj_to_meshes(parsed, named, emissive)


_LOADERS = {"trimesh": _load_trimesh, "ply": _load_ply_object, "obj": _load_obj_object}


def load_json_scene(path):
    """JsonScene.LoadFromFile: a Scene (meshes, emitters, camera, background) from a .json file."""
    with open(path) as f:
        text = f.read()
    # the reference parses with trailing commas allowed and comments skipped
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r",(\s*[\]}])", r"\1", text)
    root = json.loads(text)
    scene = Scene()
    cache = {}
    transforms = _named_transforms(root)
    _cameras(scene, root, transforms)
    bg = root.get("background")
    if bg is not None and bg["type"] == "image":
        scene.Background = EnvironmentMap(_load_rgb_image(os.path.join(os.path.dirname(path), bg["filename"]), cache))
    named, emissive = _materials(path, root, cache)
    dirname = os.path.dirname(path)
    for obj in root["objects"]:
        loader = _LOADERS.get(obj["type"])
        if loader is None:
            raise MeshLoadException(f"unknown object type '{obj['type']}'")
        meshes, emitters = loader(obj, named, emissive, dirname)
        for k, m in enumerate(meshes or []):
            m.Name = obj["name"] if k == 0 else obj["name"] + f".{k - 1:03d}"
        scene.Meshes.extend(meshes or [])
        scene.Emitters.extend(emitters or [])
    if "exposure" in root:
        scene.RecommendedExposure = float(root["exposure"])
    return scene


# ---------------------------------------------------------------------------------------------
# Wavefront .obj / .mtl (IO/ObjMesh.cs, IO/ObjConverter.cs)
# ---------------------------------------------------------------------------------------------
_RE_FLOAT = re.compile(r"([+-]?([0-9]+([.][0-9]*)?|[.][0-9]+))")
_RE_INDEX = re.compile(r"([+-]?[0-9]+)/?([+-]?[0-9]+)?/?([+-]?[0-9]+)?")


class ObjMaterial:
    def __init__(self):
        self.ambient = self.diffuse = self.specular = self.emission = RgbColor(0, 0, 0)
        self.transmittance = RgbColor(0, 0, 0)
        self.specularIndex = self.indexOfRefraction = self.transparency = self.dissolveFactor = 0.0
        self.illuminationModel = 0
        self.diffuseTexture = None


class ObjFile:
    """Parsed contents: objects -> groups -> faces (vertex/texcoord/normal index triples, with
    index 0 meaning absent), the vertex arrays with a dummy entry 0, material names (entry 0 is
    the empty name), the .mtl library, the parse errors and the file's directory."""

    def __init__(self):
        self.objects = [("", [("", [])])]
        self.vertices = [np.zeros(3, np.float32)]
        self.normals = [np.zeros(3, np.float32)]
        self.texcoords = [np.zeros(2, np.float32)]
        self.materials = [""]
        self.mtl_files = []
        self.material_lib = {}
        self.errors = []
        self.base_path = ""


def read_obj(path):
    """ObjMesh.FromFile: parses the .obj and every .mtl it names (missing .mtl files are skipped)."""
    f = ObjFile()
    f.base_path = os.path.dirname(os.path.abspath(path))
    cur_mtl = 0
    with open(path) as fh:
        for lineno, line in enumerate(fh, 1):
            line = line.strip()
            if not line or line[0] == "#":
                continue
            if line[0] == "v" and len(line) > 1:
                nums = [float(m.group(0)) for m in _RE_FLOAT.finditer(line)]
                if line[1] in " \t":
                    if len(nums) != 3:
                        f.errors.append(f"Invalid vector (line {lineno}).")
                    f.vertices.append(np.array(nums[:3], np.float32))
                elif line[1] == "n":
                    if len(nums) != 3:
                        f.errors.append(f"Invalid vector (line {lineno}).")
                    f.normals.append(np.array(nums[:3], np.float32))
                elif line[1] == "t":
                    if len(nums) != 2:
                        f.errors.append(f"Invalid vector (line {lineno}). Replaced by (0,0).")
                        nums = [0.0, 0.0]
                    f.texcoords.append(np.array(nums[:2], np.float32))
                else:
                    f.errors.append(f"Invalid vertex (line {lineno}).")
            elif line[0] == "f" and len(line) > 1 and line[1].isspace():
                idx = []
                for m in _RE_INDEX.finditer(line[1:]):
                    v = int(m.group(1))
                    t = int(m.group(2)) if m.group(2) else 0
                    n = int(m.group(3)) if m.group(3) else 0
                    idx.append([v, t, n])
                if len(idx) < 3:
                    f.errors.append(f"Invalid face (line {lineno}).")
                    continue
                for e in idx:   # relative (negative) indices count back from the current end
                    if e[0] < 0:
                        e[0] += len(f.vertices)
                    if e[1] < 0:
                        e[1] += len(f.texcoords)
                    if e[2] < 0:
                        e[2] += len(f.normals)
                if any(e[0] <= 0 or e[1] < 0 or e[2] < 0 for e in idx):
                    f.errors.append(f"Invalid indices in face definition (line {lineno} ).")
                    continue
                f.objects[-1][1][-1][1].append((cur_mtl, [tuple(e) for e in idx]))
            elif line[0] == "g" and len(line) > 1 and line[1].isspace():
                f.objects[-1][1].append((line[2:].strip(), []))
            elif line[0] == "o" and len(line) > 1 and line[1].isspace():
                f.objects.append((line[2:].strip(), [("", [])]))
            elif line.startswith("usemtl") and len(line) > 6 and line[6].isspace():
                name = line[6:].strip()
                if name not in f.materials:
                    f.materials.append(name)
                cur_mtl = f.materials.index(name)
            elif line.startswith("mtllib") and len(line) > 6 and line[6].isspace():
                f.mtl_files.append(line[6:].strip())
            elif line[0] == "s" and len(line) > 1 and line[1].isspace():
                pass
            else:
                f.errors.append(f"Unknown command '{line}' (line {lineno}).")
    for mtl in f.mtl_files:
        p = os.path.join(f.base_path, mtl)
        if os.path.exists(p):
            _read_mtl(p, f)
    return f


def _read_mtl(path, f):
    cur = None
    with open(path) as fh:
        for lineno, line in enumerate(fh, 1):
            line = line.strip()
            if not line or line[0] == "#":
                continue

            def rgb():
                nums = [float(m.group(0)) for m in _RE_FLOAT.finditer(line)]
                if len(nums) != 3:
                    f.errors.append(f"Invalid vector (line {lineno}).")
                return RgbColor(*nums[:3])

            if line.startswith("newmtl") and len(line) > 6 and line[6].isspace():
                name = line[6:].strip()
                if name in f.material_lib:
                    f.errors.append(f"Material redefinition for '{name}' (line {lineno}).")
                else:
                    f.material_lib[name] = ObjMaterial()
                cur = f.material_lib[name]
            elif line[:3] in ("Ka ", "Kd ", "Ks ", "Ke ") or line[:3] in ("Ka\t", "Kd\t", "Ks\t", "Ke\t"):
                setattr(cur, {"a": "ambient", "d": "diffuse", "s": "specular", "e": "emission"}[line[1]], rgb())
            elif line[:2] == "Ns" and line[2].isspace():
                cur.specularIndex = float(line[3:])
            elif line[:2] == "Ni" and line[2].isspace():
                cur.indexOfRefraction = float(line[3:])
            elif line[:2] == "Tf" and line[2].isspace():
                cur.transmittance = rgb()
            elif line[:2] == "Tr" and line[2].isspace():
                cur.transparency = float(line[3:])
            elif line[0] == "d" and line[1].isspace():
                cur.dissolveFactor = float(line[2:])
            elif line.startswith("illum") and line[5].isspace():
                cur.illuminationModel = int(line[6:])
            elif line.startswith("map_Kd") and line[6].isspace():
                cur.diffuseTexture = line[7:].strip()
            elif line.startswith(("map_Ka", "map_Ks", "map_Ke", "map_bump", "bump", "map_d")):
                pass   # parsed by the reference, unused by the conversion
            else:
                f.errors.append(f"Unknown command '{line}' (line {lineno}).")


def _obj_material(m, base_path, cache):
    """The GenericMaterial an .mtl entry maps to (ObjConverter.cs:61-101)."""
    if m.illuminationModel == 5:     # perfect mirror
        p = GenericMaterial.Parameters(BaseColor=TextureRgb(m.specular), SpecularTintStrength=1.0, Metallic=1.0, Roughness=TextureMono(0.0))
    elif m.illuminationModel == 7:   # perfect glass
        p = GenericMaterial.Parameters(BaseColor=TextureRgb(m.specular), Metallic=0.0, Roughness=TextureMono(0.0),
                                       IndexOfRefraction=m.indexOfRefraction, SpecularTransmittance=1.0, SpecularTintStrength=1.0)
    else:                            # treated as Phong: diffuse colour, roughness from Ns
        base = TextureRgb(m.diffuse) if not m.diffuseTexture else TextureRgb(_load_rgb_image(os.path.join(base_path, m.diffuseTexture), cache))
        rough = 1.0 if m.specularIndex == 0 else float(np.float32(1.0) / np.float32(m.specularIndex))
        p = GenericMaterial.Parameters(BaseColor=base, Roughness=TextureMono(rough), Metallic=0.5)
    return GenericMaterial(p)


def obj_to_meshes(f, material_override=None, emission_override=None):
    """ObjConverter.CreateMeshes: triangle fans per face, one mesh per (group, material) with its
    own vertex list (one entry per distinct vertex/texcoord/normal triple, texcoord v flipped)."""
    cache = {}
    dummy = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor(1, 1, 1))))
    materials, emitters_of = {}, {}
    for name in f.materials[1:]:
        m = f.material_lib.get(name)
        if m is None:
            f.errors.append(f"Cannot find material '{name}'. Replacing by dummy.")
            materials[name] = dummy
            continue
        materials[name] = _obj_material(m, f.base_path, cache)
        if np.any(m.emission.array() != 0):
            emitters_of[name] = m.emission
    meshes, emitters = [], []
    for _oname, groups in f.objects:
        tri_groups = []
        has_n = has_t = False
        empty = True
        for _gname, faces in groups:
            by_mtl = {}
            for mtl, idx in faces:
                tris = by_mtl.setdefault(mtl, [])
                has_n |= any(e[2] != 0 for e in idx)
                has_t |= any(e[1] != 0 for e in idx)
                for i in range(1, len(idx) - 1):
                    tris.append((idx[0], idx[i], idx[i + 1]))
                    empty = False
            tri_groups.append(by_mtl)
        if empty:
            continue
        for by_mtl in tri_groups:
            for mtl, tris in by_mtl.items():
                name = f.materials[mtl]
                if material_override is not None and name in material_override:
                    material = material_override[name]
                else:
                    material = materials[name]
                remap, V, N, T, I = {}, [], [], [], []
                for tri in tris:
                    for e in tri:
                        k = remap.get(e)
                        if k is None:
                            V.append(f.vertices[e[0]])
                            if has_n:
                                N.append(f.normals[e[2]])
                            if has_t:
                                uv = f.texcoords[e[1]].copy()
                                uv[1] = np.float32(1.0) - uv[1]
                                T.append(uv)
                            k = len(V) - 1
                            remap[e] = k
                        I.append(k)
                mesh = Mesh(np.array(V, np.float32), np.array(I, np.int32), shadingNormals=np.array(N, np.float32) if has_n else None,
                            textureCoordinates=np.array(T, np.float32) if has_t else None)
                mesh.Material = material
                meshes.append(mesh)
                if emission_override is not None and name in emission_override:
                    rad, glossy, exponent = emission_override[name]
                    emitters.extend(GlossyEmitter.MakeFromMesh(mesh, rad, exponent) if glossy else DiffuseEmitter.MakeFromMesh(mesh, rad))
                elif name in emitters_of:
                    emitters.extend(DiffuseEmitter.MakeFromMesh(mesh, emitters_of[name]))
    return meshes, emitters


# ---------------------------------------------------------------------------------------------
# .ply (IO/PlyFile.cs)
# ---------------------------------------------------------------------------------------------
def read_ply(path):
    """PlyFile.ParseFile + ToMesh: ascii or binary (either byte order) vertex positions with
    optional normals (nx, ny, nz) and texture coordinates (u/s, v/t), all float properties, and
    faces as 'list uchar int|uint vertex_indices'; polygons become triangle fans, faces with
    fewer than three indices are skipped.  The returned Mesh has no material."""
    with open(path, "rb") as fh:
        data = fh.read()
    end = data.find(b"end_header")
    if not data.startswith(b"ply") or end < 0:
        raise MeshLoadException(f"Trying to load invalid .ply file: {path}")
    nl = data.index(b"\n", end)
    header = data[:nl].decode("ascii", "replace").splitlines()
    body = data[nl + 1:]
    fmt, nvert, nface = "ascii", 0, 0
    props = {}
    nprops = 0
    ind_ok = False
    for line in header[1:]:
        parts = line.split()
        if not parts:
            continue
        if parts[0] == "format" and parts[1] in ("ascii", "binary_little_endian", "binary_big_endian"):
            fmt = parts[1]
        elif parts[0] == "element":
            if parts[1] == "vertex":
                nvert = int(parts[2])
            elif parts[1] == "face":
                nface = int(parts[2])
        elif parts[0] == "property":
            if parts[1] == "float":
                nm = parts[2]
                key = {"x": "x", "y": "y", "z": "z", "nx": "nx", "ny": "ny", "nz": "nz", "u": "u", "s": "u", "v": "v", "t": "v"}.get(nm)
                if key:
                    props[key] = nprops
                nprops += 1
            elif parts[1] == "list":
                if parts[2] in ("char", "uchar", "int8", "uint8") and parts[3] in ("int", "uint") and parts[4] in ("vertex_indices", "vertex_index"):
                    ind_ok = True
            else:
                nprops += 1
    if not all(k in props for k in "xyz") or not ind_ok:
        raise MeshLoadException(f"Ply file has no data: {path}")
    has_n = all(k in props for k in ("nx", "ny", "nz"))
    has_t = all(k in props for k in ("u", "v"))
    faces = []
    if fmt == "ascii":
        lines = body.decode("ascii").split("\n")
        vals = np.array([[float(x) for x in lines[i].split()[:nprops]] + [0.0] * max(0, nprops - len(lines[i].split())) for i in range(nvert)],
                        np.float32).reshape(nvert, nprops)
        for i in range(nface):
            parts = lines[nvert + i].split()
            c = int(parts[0])
            faces.append([int(x) for x in parts[1:1 + c]])
    else:
        end_ch = "<" if fmt == "binary_little_endian" else ">"
        vals = np.frombuffer(body, np.dtype(end_ch + "f4"), count=nvert * nprops).astype(np.float32).reshape(nvert, nprops)
        p = nvert * nprops * 4
        for _ in range(nface):
            c = body[p]
            faces.append(list(struct.unpack_from(end_ch + f"{c}i", body, p + 1)))
            p += 1 + 4 * c
    V = vals[:, [props["x"], props["y"], props["z"]]]
    N = vals[:, [props["nx"], props["ny"], props["nz"]]] if has_n else None
    T = vals[:, [props["u"], props["v"]]] if has_t else None
    I = []
    for fc in faces:
        if len(fc) < 3:
            continue
        for i in range(2, len(fc)):
            I += [fc[0], fc[i - 1], fc[i]]
    return Mesh(np.ascontiguousarray(V), np.array(I, np.int32), shadingNormals=None if N is None else np.ascontiguousarray(N),
                textureCoordinates=None if T is None else np.ascontiguousarray(T))
