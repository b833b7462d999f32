"""Seeded synthetic scenes for the benchmark configurations and the parity tests.

No public dataset is involved: every scene is generated from a seed with the shapes, sizes and
value distributions of the benchmark configurations.

* cornell_box:   five 2x2 diffuse quads (grey 0.725, red left, green right wall), two boxes of 12
                 triangles rotated by seeded angles in [-20, 20] degrees, a 0.5x0.5 ceiling light of
                 radiance (17, 12, 4), pinhole camera with a 40 degree field of view (36 triangles).
* sphere_field:  seeded displaced icospheres (5120 triangles each at subdivision 4) uniformly placed
                 in a 20^3 box over a ground plane, one GenericMaterial per sphere (base colour
                 U[0,1]^3, roughness U[0.05,1], metallic Bernoulli(0.3), specular transmittance 1
                 with probability 0.1), 50 emissive triangles of radiance U[5,50], and a 512x256
                 procedural HDR sky.  200 spheres give the 1M-triangle scene.
* validation:    the analytic scenes of SeeSharp.Validation (Validate_*.cs) rebuilt in this API.
"""
from __future__ import annotations

import math

import numpy as np

from .images import FrameBuffer, RgbColor, RgbImage, TextureMono, TextureRgb
from .scene import (DiffuseEmitter, DiffuseMaterial, EnvironmentMap, GenericMaterial, GlossyEmitter, Matrix4x4, Mesh, PerspectiveCamera, Scene,
                    Triangle)


def _quad(c, u, v):
    """Quad with corner c and edges u, v; face normal along cross(u, v)."""
    c, u, v = (np.asarray(x, np.float32) for x in (c, u, v))
    return np.array([c, c + u, c + u + v, c + v], np.float32), np.array([0, 1, 2, 0, 2, 3], np.int32)


def _box(center, size, angle):
    """Axis-aligned box rotated about +Y: 8 vertices, 12 outward-facing triangles."""
    hx, hy, hz = (s / 2 for s in size)
    p = np.array([[-hx, -hy, -hz], [hx, -hy, -hz], [hx, hy, -hz], [-hx, hy, -hz],
                  [-hx, -hy, hz], [hx, -hy, hz], [hx, hy, hz], [-hx, hy, hz]], np.float32)
    c, s = math.cos(angle), math.sin(angle)
    rot = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], np.float32)
    p = p @ rot.T + np.asarray(center, np.float32)
    idx = np.array([0, 2, 1, 0, 3, 2,   # back  (-z)
                    4, 5, 6, 4, 6, 7,   # front (+z)
                    0, 1, 5, 0, 5, 4,   # bottom
                    3, 7, 6, 3, 6, 2,   # top
                    0, 4, 7, 0, 7, 3,   # left
                    1, 2, 6, 1, 6, 5], np.int32)
    return p.astype(np.float32), idx


def cornell_box(width=256, height=256, seed=7):
    rng = np.random.default_rng(seed)
    sc = Scene()
    grey, red, green = RgbColor(0.725, 0.725, 0.725), RgbColor(0.63, 0.065, 0.05), RgbColor(0.14, 0.45, 0.09)

    def add(vi, col):
        m = Mesh(*vi)
        m.Material = DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(col)))
        sc.Meshes.append(m)
        return m

    add(_quad([-1, -1, 1], [2, 0, 0], [0, 0, -2]), grey)     # floor, normal +y
    add(_quad([-1, 1, -1], [2, 0, 0], [0, 0, 2]), grey)      # ceiling, normal -y
    add(_quad([-1, -1, -1], [2, 0, 0], [0, 2, 0]), grey)     # back wall, normal +z
    add(_quad([-1, -1, 1], [0, 0, -2], [0, 2, 0]), red)      # left wall, normal +x
    add(_quad([1, -1, -1], [0, 0, 2], [0, 2, 0]), green)     # right wall, normal -x
    a1, a2 = np.radians(rng.uniform(-20, 20, size=2))
    add(_box([0.35, -0.7, 0.3], [0.6, 0.6, 0.6], a1), grey)
    add(_box([-0.35, -0.4, -0.3], [0.6, 1.2, 0.6], a2), grey)
    lv, li = _quad([-0.25, 0.998, -0.25], [0.5, 0, 0], [0, 0, 0.5])
    light = Mesh(lv, li, shadingNormals=np.tile([0, -1, 0], (4, 1)))
    light.Material = DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor.Black)))
    sc.Meshes.append(light)
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(light, RgbColor(17, 12, 4)))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, 3.7], [0, 0, 0], [0, 1, 0]), 40)
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc


def cornell_box_differentiable(width=512, height=512, seed=7, tex_res=256, texture=None, roughness=(0.3, 0.6), radiance=(17, 12, 4)):
    """The differentiation configuration: the Cornell box with a GenericMaterial back wall whose
    base colour is a tex_res^2 RGB texture, a GenericMaterial with a scalar roughness on each box,
    and the ceiling light's RGB radiance.  Returns (scene, texture, box_materials, light_emitters)."""
    rng = np.random.default_rng(seed)
    sc = cornell_box(width, height, seed)
    if texture is None:
        yy, xx = np.meshgrid(np.linspace(0, 1, tex_res), np.linspace(0, 1, tex_res), indexing="ij")
        texture = np.stack([0.35 + 0.3 * np.sin(6.0 * xx + 1.0) * np.cos(4.0 * yy), 0.5 + 0.25 * np.cos(5.0 * yy + 0.5),
                            0.45 + 0.2 * np.sin(3.0 * (xx + yy))], -1) + 0.05 * rng.standard_normal((tex_res, tex_res, 3))
        texture = np.clip(texture, 0.05, 0.95).astype(np.float32)
    tex = TextureRgb(RgbImage(np.asarray(texture, np.float32)))
    back = sc.Meshes[2]
    back.TextureCoordinates = np.array([[0, 1], [1, 1], [1, 0], [0, 0]], np.float32)
    back.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=tex, Roughness=TextureMono(0.8), SpecularTintStrength=0.0))
    boxes = []
    for k, mesh in enumerate(sc.Meshes[5:7]):
        mat = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor(0.725, 0.725, 0.725)), Roughness=TextureMono(roughness[k]),
                                                         Metallic=0.3))
        mesh.Material = mat
        boxes.append(mat)
    for e in sc.Emitters:
        e.Radiance = RgbColor(*radiance)
    return sc, tex, boxes, list(sc.Emitters)


# ---------------------------------------------------------------------------------------------
# icospheres
# ---------------------------------------------------------------------------------------------
_ICO_CACHE = {}


def icosphere(level):
    """Unit icosphere by midpoint subdivision: (vertices, indices)."""
    if level in _ICO_CACHE:
        return _ICO_CACHE[level]
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    f = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
         [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = f
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        faces = nf
    out = (np.array(verts, np.float64), np.array(faces, np.int32).reshape(-1))
    _ICO_CACHE[level] = out
    return out


def _vertex_normals(V, I):
    tri = V[I.reshape(-1, 3)]
    fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    N = np.zeros_like(V)
    for k in range(3):
        np.add.at(N, I.reshape(-1, 3)[:, k], fn)
    N /= np.linalg.norm(N, axis=1, keepdims=True) + 1e-30
    return N


def procedural_sky(w=512, h=256, seed=3):
    """Lat-long HDR sky: a horizon gradient plus a small bright sun (rows top to bottom = +y down)."""
    rng = np.random.default_rng(seed)
    theta = (np.arange(h) + 0.5) / h * math.pi
    phi = (np.arange(w) + 0.5) / w * 2 * math.pi
    T, P = np.meshgrid(theta, phi, indexing="ij")
    up = np.cos(T)
    sky = np.stack([0.35 + 0.25 * np.clip(up, 0, 1), 0.45 + 0.3 * np.clip(up, 0, 1), 0.8 + 0.4 * np.clip(up, 0, 1)], -1)
    ground = np.stack([0.12, 0.1, 0.08]) * np.ones_like(sky)
    img = np.where(up[..., None] >= 0, sky, ground)
    st, sp = math.radians(rng.uniform(25, 50)), rng.uniform(0, 2 * math.pi)
    d = np.stack([np.sin(T) * np.cos(P), np.cos(T), np.sin(T) * np.sin(P)], -1)
    sd = np.array([math.sin(st) * math.cos(sp), math.cos(st), math.sin(st) * math.sin(sp)])
    cosang = d @ sd
    img = img + (cosang > math.cos(math.radians(2.5)))[..., None] * np.array([800.0, 700.0, 550.0])
    return img.astype(np.float32)


def sphere_field(num_spheres=200, width=1024, height=1024, seed=11, level=4, num_lights=50, env=True):
    rng = np.random.default_rng(seed)
    base_v, base_i = icosphere(level)
    nv = base_v.shape[0]
    sc = Scene()
    # ground plane
    gv, gi = _quad([-20, -1.5, 40], [80, 0, 0], [0, 0, -80])
    ground = Mesh(gv, gi)
    ground.Material = DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor(0.5, 0.5, 0.5))))
    sc.Meshes.append(ground)
    freq = rng.uniform(2, 6, size=(num_spheres, 3, 3))
    phase = rng.uniform(0, 2 * math.pi, size=(num_spheres, 3))
    for s in range(num_spheres):
        center = rng.uniform(0, 20, size=3)
        radius = rng.uniform(0.6, 1.4)
        disp = np.zeros(nv)
        for k in range(3):
            disp += 0.04 * np.sin(base_v @ freq[s, k] + phase[s, k])
        V = base_v * (radius * (1.0 + disp))[:, None] + center
        N = _vertex_normals(V, base_i)
        m = Mesh(V.astype(np.float32), base_i, shadingNormals=N.astype(np.float32))
        p = GenericMaterial.Parameters(
            BaseColor=TextureRgb(RgbColor(*rng.uniform(0, 1, size=3))),
            Roughness=TextureMono(rng.uniform(0.05, 1.0)),
            Metallic=float(rng.random() < 0.3),
            SpecularTransmittance=float(rng.random() < 0.1))
        m.Material = GenericMaterial(p)
        sc.Meshes.append(m)
    # emissive triangles above the field, facing down
    lv = []
    for k in range(num_lights):
        c = np.array([rng.uniform(0, 20), rng.uniform(22, 26), rng.uniform(0, 20)])
        s = rng.uniform(0.4, 0.9)
        a = rng.uniform(0, 2 * math.pi)
        p0 = c + s * np.array([math.cos(a), 0, math.sin(a)])
        p1 = c + s * np.array([math.cos(a + 2.1), 0, math.sin(a + 2.1)])
        p2 = c + s * np.array([math.cos(a + 4.2), 0, math.sin(a + 4.2)])
        n = np.cross(p1 - p0, p2 - p0)
        if n[1] > 0:
            p1, p2 = p2, p1
        lv += [p0, p1, p2]
    lights = Mesh(np.array(lv, np.float32), np.arange(3 * num_lights, dtype=np.int32))
    lights.Material = DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor.Black)))
    sc.Meshes.append(lights)
    for k in range(num_lights):
        sc.Emitters.append(DiffuseEmitter(Triangle(lights, k), RgbColor(*rng.uniform(5, 50, size=3))))
    if env:
        sc.Background = EnvironmentMap(RgbImage(procedural_sky(seed=seed + 1)))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([10, 9, -16], [10, 8, 10], [0, 1, 0]), 45)
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc


def _terrain(n, x0, z0, size, seed):
    """Heightfield of n x n quads over [x0, x0 + size] x [z0, z0 + size]: vertices (n+1)^2, UVs
    spanning [0, 1]^2, heights a seeded sum of sines around y = -1.5."""
    rng = np.random.default_rng(seed)
    g = np.linspace(0.0, 1.0, n + 1)
    U, Vv = np.meshgrid(g, g, indexing="xy")
    h = np.zeros_like(U)
    for _ in range(6):
        f = rng.uniform(2, 12, size=2)
        a = rng.uniform(0.1, 0.6)
        h += a * np.sin(2 * math.pi * (f[0] * U + rng.uniform())) * np.cos(2 * math.pi * (f[1] * Vv + rng.uniform()))
    V = np.stack([x0 + size * U, -1.5 + h, z0 + size * Vv], -1).reshape(-1, 3).astype(np.float32)
    uv = np.stack([U, 1.0 - Vv], -1).reshape(-1, 2).astype(np.float32)
    i = np.arange(n)
    a = (i[None, :] + (n + 1) * i[:, None]).reshape(-1)
    b, c, d = a + 1, a + n + 2, a + n + 1
    I = np.stack([a, c, b, a, d, c], -1).reshape(-1).astype(np.int32)  # faces point up (+y)
    return V, I, uv


def large_combined(width=1920, height=1080, seed=21, num_spheres=2000, terrain_quads=1024, tex_res=1024, num_lights=1000, views=8, level=4):
    """The large combined workload: num_spheres seeded displaced icospheres (5120 triangles each
    at subdivision 4) with one GenericMaterial each (its roughness is a parameter), a heightfield
    terrain of terrain_quads^2 quads whose GenericMaterial base colour is a tex_res^2 RGB texture
    (a parameter), num_lights emissive triangles, a procedural sky and `views` camera views
    around the field.  2000 spheres + 1024^2 quads give 12.3M triangles.
    Returns (scene, terrain texture, sphere materials, [(worldToCamera, fov)] views)."""
    rng = np.random.default_rng(seed)
    base_v, base_i = icosphere(level)
    nv = base_v.shape[0]
    sc = Scene()
    extent = 100.0
    tv, ti, tuv = _terrain(terrain_quads, -10.0, -10.0, extent, seed + 1)
    yy, xx = np.meshgrid(np.linspace(0, 1, tex_res), np.linspace(0, 1, tex_res), indexing="ij")
    tex_img = np.stack([0.3 + 0.2 * np.sin(23 * xx) * np.cos(17 * yy), 0.45 + 0.2 * np.cos(31 * yy + 1.0), 0.25 + 0.15 * np.sin(13 * (xx + yy))], -1)
    tex_img = np.clip(tex_img + 0.05 * rng.standard_normal(tex_img.shape), 0.02, 0.98).astype(np.float32)
    tex = TextureRgb(RgbImage(tex_img))
    terrain = Mesh(tv, ti, textureCoordinates=tuv)
    terrain.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=tex, Roughness=TextureMono(0.7), SpecularTintStrength=0.0))
    sc.Meshes.append(terrain)
    freq = rng.uniform(2, 6, size=(num_spheres, 3, 3))
    phase = rng.uniform(0, 2 * math.pi, size=(num_spheres, 3))
    mats = []
    for k in range(num_spheres):
        center = np.array([rng.uniform(0, 80), rng.uniform(0.0, 6.0), rng.uniform(0, 80)])
        radius = rng.uniform(0.5, 1.3)
        disp = np.zeros(nv)
        for j in range(3):
            disp += 0.04 * np.sin(base_v @ freq[k, j] + phase[k, j])
        V = base_v * (radius * (1.0 + disp))[:, None] + center
        N = _vertex_normals(V, base_i)
        m = Mesh(V.astype(np.float32), base_i, shadingNormals=N.astype(np.float32))
        mat = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor(*rng.uniform(0.05, 0.95, size=3))),
                                                         Roughness=TextureMono(rng.uniform(0.1, 0.9)), Metallic=float(rng.random() < 0.3)))
        m.Material = mat
        mats.append(mat)
        sc.Meshes.append(m)
    lv = []
    for k in range(num_lights):
        c = np.array([rng.uniform(-5, 85), rng.uniform(25, 30), rng.uniform(-5, 85)])
        sz = rng.uniform(0.5, 1.2)
        a = rng.uniform(0, 2 * math.pi)
        p0 = c + sz * np.array([math.cos(a), 0, math.sin(a)])
        p1 = c + sz * np.array([math.cos(a + 2.1), 0, math.sin(a + 2.1)])
        p2 = c + sz * np.array([math.cos(a + 4.2), 0, math.sin(a + 4.2)])
        if np.cross(p1 - p0, p2 - p0)[1] > 0:
            p1, p2 = p2, p1
        lv += [p0, p1, p2]
    lights = Mesh(np.array(lv, np.float32), np.arange(3 * num_lights, dtype=np.int32))
    lights.Material = DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor.Black)))
    sc.Meshes.append(lights)
    for k in range(num_lights):
        sc.Emitters.append(DiffuseEmitter(Triangle(lights, k), RgbColor(*rng.uniform(5, 40, size=3))))
    sc.Background = EnvironmentMap(RgbImage(procedural_sky(seed=seed + 2)))
    cams = []
    for v in range(views):
        a = 2 * math.pi * v / views + 0.3
        eye = [40 + 55 * math.cos(a), rng.uniform(12, 22), 40 + 55 * math.sin(a)]
        cams.append((Matrix4x4.CreateLookAt(eye, [40, 0, 40], [0, 1, 0]), 50.0))
    sc.Camera = PerspectiveCamera(cams[0][0], cams[0][1])
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc, tex, mats, cams


def sphere_field_for_triangles(num_triangles, **kw):
    return sphere_field(num_spheres=max(1, int(round(num_triangles / 5120))), **kw)


# ---------------------------------------------------------------------------------------------
# SeeSharp.Validation scenes (Validate_*.cs), rebuilt in this API
# ---------------------------------------------------------------------------------------------
def _ground(z=-2.0):
    return Mesh([[-10, -10, z], [10, -10, z], [10, 10, z], [-10, 10, z]], [0, 1, 2, 0, 2, 3])


def _small_emitter(depth, normal_z, offset=(0.0, 0.0), size=0.1):
    ox, oy = offset
    return Mesh([[-size + ox, -size + oy, depth], [size + ox, -size + oy, depth], [size + ox, size + oy, depth], [-size + ox, size + oy, depth]],
                [0, 1, 2, 0, 2, 3], shadingNormals=[[0, 0, normal_z]] * 4)


def _black():
    return DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor.Black)))


def validate_direct_illum(width=512, height=512):
    """Validate_DirectIllum.cs:19-64 (10 spp, max depth 2)."""
    sc = Scene()
    g = _ground()
    g.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor.White), Roughness=TextureMono(0.5)))
    e = _small_emitter(-1.0, -1)
    e.Material = _black()
    sc.Meshes += [g, e]
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(e, RgbColor.White * 1000))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, 0], [0, 0, -1], [0, 1, 0]), 40)
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc, 10, 2


def validate_direct_transmit(width=512, height=512):
    """Validate_DirectTransmit.cs (10 spp, max depth 2)."""
    sc = Scene()
    g = _ground()
    g.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor.White * 0.8), Roughness=TextureMono(1.0), Anisotropic=1.0,
                                                            IndexOfRefraction=1.45, Metallic=0.0, SpecularTransmittance=1.0,
                                                            SpecularTintStrength=0.0))
    e = _small_emitter(-4.0, 1)
    e.Material = _black()
    sc.Meshes += [g, e]
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(e, RgbColor.White * 1000))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, 0], [0, 0, -1], [0, 1, 0]), 40)
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc, 10, 2


def validate_multi_light(width=512, height=512):
    """Validate_MultiLight.cs (10 spp, max depth 2)."""
    sc = Scene()
    g = _ground()
    g.Material = DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor.White)))
    sc.Meshes.append(g)
    for ox in (-1.0, 1.0):
        e = _small_emitter(-1.0, -1, (ox, 0.0))
        e.Material = _black()
        sc.Meshes.append(e)
        sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(e, RgbColor.White * 1000))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, 0], [0, 0, -1], [0, 1, 0]), 40)
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc, 10, 2


def validate_glossy_light(width=512, height=512):
    """Validate_GlossyLight.cs (10 spp, max depth 2)."""
    sc = Scene()
    g = _ground(0.0)
    g.Material = DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor.White), Transmitter=True))
    e = _small_emitter(-1.0, 1)
    e.Material = _black()
    sc.Meshes += [g, e]
    sc.Emitters.extend(GlossyEmitter.MakeFromMesh(e, RgbColor.White * 1000, 200))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, 2], [0, 0, -1], [0, 1, 0]), 40)
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc, 10, 2


def validate_single_bounce(width=512, height=512):
    """Validate_SingleBounce.cs (10 spp, max depth 3)."""
    sc = Scene()
    g = _ground()
    g.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor.White)))
    e = _small_emitter(1.0, 1)
    e.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor.Black)))
    r = Mesh([[-10, -10, 2], [10, -10, 2], [10, 10, 2], [-10, 10, 2]], [0, 1, 2, 0, 2, 3], shadingNormals=[[0, 0, 1]] * 4)
    r.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor.White)))
    sc.Meshes += [g, e, r]
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(e, RgbColor.White * 1000))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, 0], [0, 0, -1], [0, 1, 0]), 40)
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc, 10, 3


def validate_single_bounce_glossy(width=512, height=512):
    """Validate_SingleBounceGlossy.cs (32 spp, max depth 3): a rough (0.5) transmissive plane in
    front of a rough reflector, lit by a 0.1-area quad of power 500 facing -z."""
    sc = Scene()
    a = Mesh([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], [0, 1, 2, 0, 2, 3])
    a.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor.White), Roughness=TextureMono(0.5),
                                                           SpecularTransmittance=1.0))
    b = Mesh([[-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], [0, 1, 2, 0, 2, 3])
    b.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor.White), Roughness=TextureMono(0.5)))
    area = np.float32(0.1)
    pos = float(np.sqrt(area) / np.float32(2))
    l = Mesh([[-pos, -pos, 11], [pos, -pos, 11], [pos, pos, 11], [-pos, pos, 11]], [0, 1, 2, 0, 2, 3], shadingNormals=[[0, 0, -1]] * 4)
    l.Material = _black()
    sc.Meshes += [a, b, l]
    radiance = float(np.float32(500) / (np.float32(math.pi) * area))
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(l, RgbColor.White * radiance))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, -1], [0, 0, 0], [0, 1, 0]), 45)
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc, 32, 3


def validate_cornell_box(width=512, height=512, data_dir=None):
    """Validate_CornellBox.cs: Data/Scenes/CornellBox/CornellBox.json, 512 x 512, 8 spp, max depth 5."""
    from . import sceneio
    sc = sceneio.load_json_scene(_scene_file(data_dir, "CornellBox/CornellBox.json"))
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc, 8, 5


def env_lit_box(width=512, height=512, seed=5):
    """A diffuse ground and a GenericMaterial box lit only by a seeded procedural sky (lat-long
    environment map, 128 x 64): an environment-lighting workload for the tests."""
    sc = Scene()
    g = Mesh([[-10, -1, -10], [10, -1, -10], [10, -1, 10], [-10, -1, 10]], [0, 2, 1, 0, 3, 2])
    g.Material = DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor(0.8, 0.8, 0.8))))
    bv, bi = _box([0, -0.5, 0], [1, 1, 1], 0.3)
    b = Mesh(bv, bi)
    b.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor(0.7, 0.3, 0.2)), Roughness=TextureMono(0.3)))
    sc.Meshes += [g, b]
    sc.Background = EnvironmentMap(RgbImage(procedural_sky(128, 64, seed=seed)))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 1, 4], [0, -0.3, 0], [0, 1, 0]), 45)
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc


def _scene_file(data_dir, rel):
    import os
    if data_dir is None:
        raise ValueError(f"this Validation scene loads {rel}: pass data_dir, the directory that holds SeeSharp's Data/Scenes files")
    return os.path.join(data_dir, rel)


def validate_environment(width=512, height=512, data_dir=None):
    """Validate_Environment.cs: Data/Scenes/simplebackground.json (lit by Data/Scenes/sunsky.exr),
    512 x 512, 10 spp, max depth 5.  data_dir: the directory holding the reference's Data/Scenes files."""
    from . import sceneio
    sc = sceneio.load_json_scene(_scene_file(data_dir, "simplebackground.json"))
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc, 10, 5


def validate_textures(width=700, height=500, data_dir=None):
    """Validate_Textures.cs: Data/Scenes/TextureTest/TextureTest.json (an OBJ mesh with a PNG
    texture), 700 x 500, 8 spp, max depth 5."""
    from . import sceneio
    sc = sceneio.load_json_scene(_scene_file(data_dir, "TextureTest/TextureTest.json"))
    sc.FrameBuffer = FrameBuffer(width, height)
    return sc, 8, 5


# SeeSharp.Validation's factories (Validate_*.cs) by name.  Each takes (width, height) and returns
# (scene, SamplesPerPixel, MaxDepth); the ones that load the reference's scene files also take
# data_dir, the directory that holds SeeSharp's Data/Scenes files.
VALIDATION_SCENES = {
    "DirectIllumination": validate_direct_illum,
    "DirectIllumTransmit": validate_direct_transmit,
    "MultiLight": validate_multi_light,
    "GlossyLight": validate_glossy_light,
    "SingleBounce": validate_single_bounce,
    "SingleBounceGlossy": validate_single_bounce_glossy,
    "Environment": validate_environment,
    "TextureTest": validate_textures,
    "CornellBox": validate_cornell_box,
}
SCENE_FILE_VALIDATIONS = ("Environment", "TextureTest", "CornellBox")
