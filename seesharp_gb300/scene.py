"""Scene model mirroring SeeSharp's Scene, Mesh, materials, emitters, background and camera.

The classes carry the same names, fields and validation rules as the reference
(Scene.cs, Geometry/Mesh.cs, Geometry/Triangle.cs, Shading/Materials/*.cs, Shading/Emitters/*.cs,
Shading/Background/EnvironmentMap.cs, Cameras/PerspectiveCamera.cs).  Scene.Prepare() uploads the
scene to the GPU through libsst (sst_scene_* in include/sst.h); there is no CPU renderer behind it.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _native
from .images import MonochromeImage, RgbColor, RgbImage, TextureMono, TextureRgb


class InvalidOperationException(RuntimeError):
    """Raised where the reference throws InvalidOperationException (Scene.cs:104-105)."""


class ArgumentException(ValueError):
    """Raised where the reference throws ArgumentException (Triangle.cs:32-33, Camera.cs:40)."""


def _f32(x):
    return np.float32(x)


class Matrix4x4:
    """System.Numerics.Matrix4x4 constructors used by SeeSharp, as float32 (4, 4) arrays.

    Row-vector convention: a point p maps to p @ M (the translation is in the last row).
    """

    @staticmethod
    def Identity():
        return np.eye(4, dtype=np.float32)

    @staticmethod
    def CreateLookAt(cameraPosition, cameraTarget, cameraUpVector):
        """Right-handed look-at matrix (world to camera), as documented for System.Numerics."""
        p = np.asarray(cameraPosition, np.float32)
        t = np.asarray(cameraTarget, np.float32)
        up = np.asarray(cameraUpVector, np.float32)
        z = p - t
        z = z / np.float32(math.sqrt(float(np.dot(z, z))))
        x = np.cross(up, z).astype(np.float32)
        x = x / np.float32(math.sqrt(float(np.dot(x, x))))
        y = np.cross(z, x).astype(np.float32)
        m = np.zeros((4, 4), np.float32)
        m[0:3, 0] = x
        m[0:3, 1] = y
        m[0:3, 2] = z
        m[3, 0] = -np.dot(x, p)
        m[3, 1] = -np.dot(y, p)
        m[3, 2] = -np.dot(z, p)
        m[3, 3] = 1
        return m

    @staticmethod
    def CreateTranslation(x, y, z):
        m = np.eye(4, dtype=np.float32)
        m[3, 0:3] = (x, y, z)
        return m

    @staticmethod
    def CreateRotationY(radians):
        c, s = math.cos(radians), math.sin(radians)
        m = np.eye(4, dtype=np.float32)
        m[0, 0] = c
        m[0, 2] = -s
        m[2, 0] = s
        m[2, 2] = c
        return m

    @staticmethod
    def CreateScale(sx, sy=None, sz=None):
        sy = sx if sy is None else sy
        sz = sx if sz is None else sz
        return np.diag(np.array([sx, sy, sz, 1], np.float32))

    @staticmethod
    def CreateFromYawPitchRoll(yaw, pitch, roll):
        """Rotation by roll about z, then pitch about x, then yaw about y (row vectors), built
        through the unit quaternion of the three half-angle rotations."""
        sr, cr = math.sin(roll * 0.5), math.cos(roll * 0.5)
        sp, cp = math.sin(pitch * 0.5), math.cos(pitch * 0.5)
        sy, cy = math.sin(yaw * 0.5), math.cos(yaw * 0.5)
        x = cy * sp * cr + sy * cp * sr
        y = sy * cp * cr - cy * sp * sr
        z = cy * cp * sr - sy * sp * cr
        w = cy * cp * cr + sy * sp * sr
        m = np.eye(4, dtype=np.float64)
        m[0, 0] = 1 - 2 * (y * y + z * z)
        m[0, 1] = 2 * (x * y + z * w)
        m[0, 2] = 2 * (x * z - y * w)
        m[1, 0] = 2 * (x * y - z * w)
        m[1, 1] = 1 - 2 * (z * z + x * x)
        m[1, 2] = 2 * (y * z + x * w)
        m[2, 0] = 2 * (x * z + y * w)
        m[2, 1] = 2 * (y * z - x * w)
        m[2, 2] = 1 - 2 * (y * y + x * x)
        return m.astype(np.float32)

    @staticmethod
    def Invert(m):
        """(True, inverse) or (False, NaN matrix) like Matrix4x4.Invert."""
        m = np.asarray(m, np.float64)
        if abs(np.linalg.det(m)) < 1e-30:
            return False, np.full((4, 4), np.nan, np.float32)
        return True, np.linalg.inv(m).astype(np.float32)


# ---------------------------------------------------------------------------------------------
# Geometry
# ---------------------------------------------------------------------------------------------
class Mesh:
    """A triangle mesh (Geometry/Mesh.cs:28-41): vertices (N, 3), indices (3T,) or (T, 3),
    optional per-vertex shading normals (N, 3) and texture coordinates (N, 2)."""

    def __init__(self, vertices, indices, shadingNormals=None, textureCoordinates=None):
        self.Vertices = np.ascontiguousarray(np.asarray(vertices, np.float32).reshape(-1, 3))
        self.Indices = np.ascontiguousarray(np.asarray(indices, np.int32).reshape(-1))
        if self.Indices.size % 3 != 0:
            raise ArgumentException("index count must be a multiple of three")
        nv = self.Vertices.shape[0]
        if self.Indices.size and (self.Indices.min() < 0 or self.Indices.max() >= nv):
            raise ArgumentException("vertex index out of range")
        self.ShadingNormals = None if shadingNormals is None else np.ascontiguousarray(np.asarray(shadingNormals, np.float32).reshape(nv, 3))
        self.TextureCoordinates = None if textureCoordinates is None else np.ascontiguousarray(
            np.asarray(textureCoordinates, np.float32).reshape(nv, 2))
        self.Material = None
        self.Name = None

    @property
    def NumFaces(self):
        return self.Indices.size // 3

    @property
    def NumVertices(self):
        return self.Vertices.shape[0]

    def FaceAreas(self):
        """|cross(v2 - v1, v3 - v1)| * 0.5 per face, in float32 (Mesh.cs:32-39)."""
        tri = self.Vertices[self.Indices.reshape(-1, 3)]
        n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]).astype(np.float32)
        return (np.sqrt((n * n).sum(axis=1, dtype=np.float32)) * np.float32(0.5)).astype(np.float32)

    @property
    def SurfaceArea(self):
        return float(self.FaceAreas().sum(dtype=np.float32))


class Triangle:
    """View of one face of a mesh (Geometry/Triangle.cs:22-36)."""

    def __init__(self, mesh, faceIndex):
        self.Mesh = mesh
        self.FaceIndex = int(faceIndex)
        i = mesh.Indices[3 * self.FaceIndex:3 * self.FaceIndex + 3]
        v1, v2, v3 = mesh.Vertices[i[0]], mesh.Vertices[i[1]], mesh.Vertices[i[2]]
        n = np.cross(v2 - v1, v3 - v1).astype(np.float32)
        area = np.float32(math.sqrt(float(np.dot(n, n)))) * np.float32(0.5)
        if area == 0:
            raise ArgumentException("Zero-area triangles cannot be emitters")
        self.SurfaceArea = float(area)


# ---------------------------------------------------------------------------------------------
# Materials
# ---------------------------------------------------------------------------------------------
class Material:
    Name = None


class DiffuseMaterial(Material):
    """Lambertian reflector or 50/50 reflector-transmitter (Shading/Materials/DiffuseMaterial.cs)."""

    class Parameters:
        def __init__(self, BaseColor=None, Transmitter=False):
            self.BaseColor = BaseColor if BaseColor is not None else TextureRgb(RgbColor.White)
            self.Transmitter = bool(Transmitter)

    def __init__(self, parameters=None):
        self.MaterialParameters = parameters if parameters is not None else DiffuseMaterial.Parameters()


class GenericMaterial(Material):
    """Disney-style material (Shading/Materials/GenericMaterial.cs:25-61 for the defaults)."""

    class Parameters:
        def __init__(self, BaseColor=None, Roughness=None, Metallic=0.0, SpecularTintStrength=1.0, Anisotropic=0.0,
                     SpecularTransmittance=0.0, IndexOfRefraction=1.45):
            self.BaseColor = BaseColor if BaseColor is not None else TextureRgb(RgbColor.White)
            self.Roughness = Roughness if Roughness is not None else TextureMono(0.5)
            self.Metallic = float(Metallic)
            self.SpecularTintStrength = float(SpecularTintStrength)
            self.Anisotropic = float(Anisotropic)
            self.SpecularTransmittance = float(SpecularTransmittance)
            self.IndexOfRefraction = float(IndexOfRefraction)

    def __init__(self, parameters=None):
        self.MaterialParameters = parameters if parameters is not None else GenericMaterial.Parameters()


# ---------------------------------------------------------------------------------------------
# Emitters and background
# ---------------------------------------------------------------------------------------------
class Emitter:
    def __init__(self, triangle, radiance):
        self.Triangle = triangle
        self.Radiance = RgbColor(radiance)

    @property
    def Mesh(self):
        return self.Triangle.Mesh

    exponent = -1.0


class DiffuseEmitter(Emitter):
    """Constant radiance over the hemisphere of the shading normal (Shading/Emitters/DiffuseEmitter.cs)."""

    @staticmethod
    def MakeFromMesh(mesh, radiance):
        out = []
        for i in range(mesh.NumFaces):
            try:
                out.append(DiffuseEmitter(Triangle(mesh, i), radiance))
            except ArgumentException:
                continue
        return out


class GlossyEmitter(Emitter):
    """Cosine-lobe emission (Shading/Emitters/GlossyEmitter.cs)."""

    def __init__(self, triangle, radiance, exponent):
        super().__init__(triangle, radiance)
        self.exponent = float(exponent)

    @staticmethod
    def MakeFromMesh(mesh, radiance, exponent):
        out = []
        for i in range(mesh.NumFaces):
            try:
                out.append(GlossyEmitter(Triangle(mesh, i), radiance, exponent))
            except ArgumentException:
                continue
        return out


class EnvironmentMap:
    """Lat-long HDR background with luminance-proportional sampling (Shading/Background/EnvironmentMap.cs)."""

    def __init__(self, image):
        if not isinstance(image, RgbImage):
            image = RgbImage(np.asarray(image, np.float32))
        self.Image = image


# ---------------------------------------------------------------------------------------------
# Camera
# ---------------------------------------------------------------------------------------------
class PerspectiveCamera:
    """Pinhole camera (Cameras/PerspectiveCamera.cs); worldToCamera is a Matrix4x4 array."""

    def __init__(self, worldToCamera, verticalFieldOfView, lensRadius=0.0, focalDistance=0.0):
        m = np.asarray(worldToCamera, np.float32).reshape(4, 4)
        if abs(np.linalg.det(m.astype(np.float64))) < 1e-30:
            raise ArgumentException("World to camera transform must be invertible.")
        if lensRadius != 0:
            raise NotImplementedError("thin-lens depth of field is not supported by the reference either")
        self.WorldToCamera = m
        self.VerticalFieldOfView = float(verticalFieldOfView)
        self.Width = 0
        self.Height = 0

    def UpdateResolution(self, width, height):
        self.Width, self.Height = int(width), int(height)

    @property
    def Position(self):
        inv = np.linalg.inv(self.WorldToCamera.astype(np.float64))
        return inv[3, 0:3].astype(np.float32)


# ---------------------------------------------------------------------------------------------
# Scene
# ---------------------------------------------------------------------------------------------
class Scene:
    """Scene container (Scene.cs).  Prepare() validates and commits it to the GPU."""

    def __init__(self, device=0):
        self.Meshes = []
        self.Emitters = []
        self.Background = None
        self.Camera = None
        self.FrameBuffer = None
        self.ValidationErrorMessages = []
        self.device = device
        self._native = None
        self._emitter_index = {}

    @property
    def IsValid(self):
        """Scene.IsValid (Scene.cs:170-197)."""
        msgs = []
        if self.FrameBuffer is None:
            msgs.append("Framebuffer not set.")
        if self.Camera is None:
            msgs.append("Camera not set.")
        if not self.Meshes:
            msgs.append("No meshes in the scene.")
        for idx, m in enumerate(self.Meshes):
            if m.Material is None:
                msgs.append(f"Mesh[{idx}] does not have a material.")
        if len(self.Emitters) == 0 and self.Background is None:
            msgs.append("No emitters and no background in the scene.")
        self.ValidationErrorMessages = msgs
        return not msgs

    def Prepare(self):
        """Scene.Prepare (Scene.cs:103-164): validate, upload, build the BVH, emitter table and
        environment-map sampling tables, and set the camera resolution."""
        if not self.IsValid:
            raise InvalidOperationException("Cannot finalize an invalid scene.")
        self.Camera.UpdateResolution(self.FrameBuffer.Width, self.FrameBuffer.Height)
        self.Dispose()
        ctx = _native.default_context(self.device)
        self._native = _native.SceneHandle(ctx)
        sc = self._native
        mesh_ids = {}
        mat_ids = {}
        for m in self.Meshes:
            mat = m.Material
            if id(mat) not in mat_ids:
                mat_ids[id(mat)] = sc.add_material(mat)
            mesh_ids[id(m)] = sc.add_mesh(m, mat_ids[id(mat)])
        self._mesh_ids = mesh_ids
        self._mat_ids = mat_ids
        # Emitters: consecutive runs with the same mesh, radiance and lobe become one call.
        self._emitter_index = {}
        run = []

        def flush():
            if not run:
                return
            e0 = run[0]
            faces = np.array([e.Triangle.FaceIndex for e in run], np.int32)
            first = sc.add_emitters(mesh_ids[id(e0.Mesh)], faces, e0.Radiance.array(), e0.exponent)
            for k, e in enumerate(run):
                self._emitter_index[id(e)] = first + k
            run.clear()

        for e in self.Emitters:
            if id(e.Mesh) not in mesh_ids:
                raise InvalidOperationException("emitter on a mesh that is not part of the scene")
            if run and not (run[0].Mesh is e.Mesh and run[0].Radiance == e.Radiance and run[0].exponent == e.exponent):
                flush()
            run.append(e)
        flush()
        if self.Background is not None:
            sc.set_envmap(self.Background.Image.data)
        sc.set_camera(self.Camera.WorldToCamera, self.Camera.VerticalFieldOfView)
        sc.commit(self.FrameBuffer.Width, self.FrameBuffer.Height)

    def QueryEmitter(self, mesh, primId):
        """Scene.QueryEmitter (Scene.cs:204-210): the emitter on (mesh, face) or None."""
        for e in self.Emitters:
            if e.Mesh is mesh and e.Triangle.FaceIndex == int(primId):
                return e
        return None

    def GetEmitterIndex(self, emitter):
        return self.Emitters.index(emitter)

    @property
    def native(self):
        if self._native is None:
            raise InvalidOperationException("scene is not prepared")
        return self._native

    def Dispose(self):
        if self._native is not None:
            self._native.close()
            self._native = None

    def __del__(self):
        try:
            self.Dispose()
        except Exception:
            pass
