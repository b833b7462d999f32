"""Pins the oracle against the reference's own known-answer tests (SeeSharp.Tests).

Each test restates one xUnit test of the reference (file:line given) with the same inputs and
the same tolerance (Assert.Equal(a, b, p) == agreement to p decimal places).  CPU only.
"""
import math

import numpy as np
import pytest

from oracle import pyoracle as O
from seesharp_gb300 import (DiffuseEmitter, DiffuseMaterial, FrameBuffer, GenericMaterial, GlossyEmitter, Matrix4x4, Mesh,
                            PerspectiveCamera, RgbColor, RgbImage, Scene, TextureMono, TextureRgb, EnvironmentMap)


def eq(a, b, places):
    """xUnit Assert.Equal(expected, actual, precision): equal after rounding to `places` decimals."""
    return round(float(a), places) == round(float(b), places)


def quad_mesh(z=0.0):
    return Mesh([[-1, -1, z], [1, -1, z], [1, 1, z], [-1, 1, z]], [0, 1, 2, 0, 2, 3])


def material_scene(material):
    """One quad with the material, so the oracle holds it as material 0."""
    sc = Scene()
    m = quad_mesh()
    m.Material = material
    sc.Meshes.append(m)
    return O.OracleScene.from_scene(sc, commit=False)


# Dummy hit used by Material_Diffuse/Material_Generic: position 0, normal +Z, no shading normals
# (so the shading normal is the face normal), uv = barycentrics (0.5, 0.2).
DUMMY = np.array([0, 0, 0, 0, 0, 1, 0, 0, 1, 0.5, 0.2], np.float32)


def norm(v):
    v = np.asarray(v, np.float32)
    return v / np.float32(math.sqrt(float(np.dot(v, v))))


# ---- Camera: SeeSharp.Tests/Core/Camera/Perspective_Rays.cs:8-122 ----
def make_test_camera_scene():
    sc = Scene()
    m = quad_mesh(10.0)
    m.Material = DiffuseMaterial()
    sc.Meshes.append(m)
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, 0], [0, 0, 10], [0, 1, 0]), 90)
    sc.FrameBuffer = FrameBuffer(3, 3)
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(m, RgbColor.White))
    return O.OracleScene.from_scene(sc)


@pytest.mark.parametrize("film,expect", [
    ((0, 0), (1, 1, 1)),          # Directions_TopLeft :20-39
    ((1.5, 1.5), (0, 0, 1)),      # Directions_Center :41-59
    ((0, 1.5), (1, 0, 1)),        # Directions_Left :61-80
    ((3, 1.5), (-1, 0, 1)),       # Directions_Right :82-101
    ((3, 3), (-1, -1, 1)),        # Directions_BottomRight :103-122
])
def test_perspective_rays(film, expect):
    o = make_test_camera_scene()
    org, d = o.camera_ray(*film)
    assert np.all(org == 0)
    e = np.array(expect, np.float64)
    e = e / np.linalg.norm(e)
    for k in range(3):
        assert eq(e[k], d[k], 3), (d, e)


# ---- Material_Diffuse.cs:4-212 ----
def test_diffuse_no_light_leaks():
    o = material_scene(DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor(1, 1, 1)))))
    val, pdf = o.material_eval(0, DUMMY, [0, 0, 1], [0, 0, -1])
    assert pdf[0] == 0 and pdf[1] == 0
    assert np.all(val == 0)


def test_diffuse_forward_reverse():
    o = material_scene(DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor(1, 1, 1)))))
    out, inn = np.array([0, 0, 1], np.float32), norm([0, 1, 1])
    _, (f1, r1) = o.material_eval(0, DUMMY, out, inn)
    _, (r2, f2) = o.material_eval(0, DUMMY, inn, out)
    assert eq(r1, r2, 3) and eq(f1, f2, 3)
    d, pdf, w = o.material_sample(0, DUMMY, out, 0.4, 0.2, 0.7)
    _, (fs, rs) = o.material_eval(0, DUMMY, out, d)
    assert eq(pdf[0], fs, 3) and eq(pdf[1], rs, 3)


@pytest.mark.parametrize("color", [(1, 1, 1), (1, 0, 0)])
def test_diffuse_albedo(color):
    """Albedo_ShouldBeWhite :81-119 / Albedo_ShouldBeRed :121-159."""
    o = material_scene(DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor(*color)))))
    retro, _ = o.material_eval(0, DUMMY, [0, 0, 1], [0, 0, 1])
    _, _, w = o.material_sample(0, DUMMY, [0, 0, 1], 0.3, 0.25, 0.8)
    for k in range(3):
        assert eq(color[k] / math.pi, retro[k], 3)
        assert eq(color[k], w[k], 3)


def test_diffuse_edge_cases():
    """EdgeCases_ShouldNotCauseOutliers :161-212."""
    o = material_scene(DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor(1, 1, 1)))))
    eps = np.float32(1.4e-45)
    prims = [(0, 0), (0, 1), (1, 0), (1, 1), (eps, eps), (eps, 1 - eps), (1 - eps, eps), (1 - eps, 1 - eps)]
    for p in prims:
        _, pdf, w = o.material_sample(0, DUMMY, [0, 0, 1], 0.5, *p)
        target = 0.0 if pdf[0] == 0 else 1.0
        for k in range(3):
            assert eq(target, w[k], 3), (p, pdf, w)


# ---- Material_Generic.cs:11-121 ----
GENERIC_CASES = [(0, 0, 1, 0, 1, 1), (1, 0, 1, 0, 1, 1), (1, 0, 1, 1, 0, -1)]


def smape_below(e, a, thr=0.005):
    if e == a:
        return True
    return abs(e - a) / (0.5 * (abs(e) + abs(a))) < thr


def generic_test_material():
    return GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor(1, 1, 1)), Roughness=TextureMono(0.2),
                                                      SpecularTransmittance=0.8))


@pytest.mark.parametrize("case", GENERIC_CASES)
def test_generic_pdfs_consistent(case):
    """Pdfs_ShouldBeConsistent :11-44."""
    o = material_scene(generic_test_material())
    out, inn = norm(case[:3]), norm(case[3:])
    _, (f1, r1) = o.material_eval(0, DUMMY, out, inn)
    _, (r2, f2) = o.material_eval(0, DUMMY, inn, out)
    assert smape_below(r1, r2) and smape_below(f1, f2), (f1, r1, f2, r2)
    d, pdf, w = o.material_sample(0, DUMMY, out, 0.4, 0.2, 0.7)
    _, (fs, rs) = o.material_eval(0, DUMMY, out, d)
    assert eq(pdf[0], fs, 3) and eq(pdf[1], rs, 3)


@pytest.mark.parametrize("case", GENERIC_CASES)
def test_generic_component_pdfs(case):
    """ComponentPdfs_ShouldBeConsistent :46-121."""
    o = material_scene(generic_test_material())
    out, inn = norm(case[:3]), norm(case[3:])
    _, (fwd, rev), c = o.material_eval(0, DUMMY, out, inn, components=True)
    n = int(c[0])
    assert eq(fwd, sum(c[1 + k] * c[4 + k] for k in range(n)), 3)
    assert eq(rev, sum(c[7 + k] * c[10 + k] for k in range(n)), 3)
    _, pdf, _, c = o.material_sample(0, DUMMY, out, 0.4, 0.2, 0.7, components=True)
    n = int(c[0])
    assert eq(pdf[0], sum(c[1 + k] * c[4 + k] for k in range(n)), 3)
    assert eq(pdf[1], sum(c[7 + k] * c[10 + k] for k in range(n)), 3)


# ---- TrowbridgeReitz_CorrectValues.cs:5-49 ----
def test_ggx_ndf_values():
    ax, ay = 0.5, 0.3
    assert eq(1 / (math.pi * ax * ay), O.ggx_D(ax, ay, [0, 0, 1]), 4)
    assert eq(0.0, O.ggx_D(ax, ay, [1, 0, 0]), 4)


def test_ggx_sample_corners_finite():
    ax, ay = 0.5, 0.3
    s2 = math.sqrt(2)
    for o, u in [([0, 0, 1], (0, 1)), ([s2, 0, s2], (1, 0)), ([0, 0, 1], (1, 0))]:
        assert np.all(np.isfinite(O.ggx_sample(ax, ay, o, *u)))


# ---- ShadingSpace_Setup_Transform.cs:6-35 ----
def test_shading_space():
    s = O.world_to_shading(norm([1, 1, 0]), norm([-1, -1, 0]))
    assert s[0] == 0 and s[1] == 0 and eq(-1, s[2], 4)
    s = O.world_to_shading(np.array([1, 1, 0], np.float32), [0, 0, 1])
    assert s[2] == 0
    n, w = norm([1, 5, 0]), norm([1, 6, 2])
    w2 = O.shading_to_world(n, O.world_to_shading(n, w))
    for k in range(3):
        assert eq(w[k] / np.linalg.norm(w), w2[k], 4)


# ---- PiecewiseConstant_DistributionTest.cs:8-97 ----
def test_pwc_probabilities_and_borders():
    w = [1, 1, 2, 2]
    _, _, prob = O.pwc(w, [0.5])
    for k, e in enumerate([1 / 6, 1 / 6, 2 / 6, 2 / 6]):
        assert eq(e, prob[k], 3)
    idx, rel, _ = O.pwc(w, [0.0, 1.0, 0.999, 0.0001])
    assert idx[0] == 0 and eq(0.0, rel[0], 6)
    assert idx[1] == 3 and eq(1.0, rel[1], 6)
    assert idx[2] == 3 and eq(0.999, rel[2], 2)
    assert idx[3] == 0 and eq(0.0001 * 6, rel[3], 6)


def test_pwc_asymptotic_and_uniform_within():
    w = [1, 1, 2, 2]
    us = []
    u = np.float32(0)
    while u < 1:
        us.append(u)
        u = np.float32(u + np.float32(1 / 100))
    idx, _, _ = O.pwc(w, us)
    counts = np.bincount(idx, minlength=4) * 6 / 100
    for k, e in enumerate([1, 1, 2, 2]):
        assert eq(e, counts[k], 1)
    # the reference accumulates u in float: for (float u = 0; u < 1; u += 1f / 1000)
    us = []
    u = np.float32(0)
    while u < 1:
        us.append(u)
        u = np.float32(u + np.float32(1 / 1000))
    _, rel, _ = O.pwc(w, us)
    cells = np.clip((rel * np.float32(1000)).astype(np.float32), 0, 1000).astype(int)
    assert len(set(cells.tolist())) > 800


def test_pwc_singularity():
    idx, _, _ = O.pwc([283, 0, 0, 0, 0], [0.0, 1.0, 0.999, 0.0001, 0.1, 0.8])
    assert np.all(idx == 0)


# ---- SampleWarp_*.cs ----
@pytest.mark.parametrize("u", [(0.1, 0.1), (0.1, 0.9), (0.25, 0.25)])
def test_warp_triangle_inverse(u):
    """SampleWarp_Triangle.cs:7-31."""
    _, inv = O.warp_triangle(*u)
    assert eq(u[0], inv[0], 4) and eq(u[1], inv[1], 4)


def test_warp_sphere_and_coshemi_inverse():
    """SampleWarp_Sphere.cs:7-14, SampleWarp_Spherical.cs."""
    for u in [(0.3, 0.8), (0.7, 0.1), (0.5, 0.5)]:
        d, inv = O.warp_sphere(*u)
        assert eq(1.0, np.linalg.norm(d), 4)
        assert eq(u[0], inv[0], 3) and eq(u[1], inv[1], 3)
        d, pdf, inv = O.warp_coshemi(*u)
        assert eq(d[2] / math.pi, pdf, 5)
        assert eq(u[0], inv[0], 3) and eq(u[1], inv[1], 3)


def test_warp_disc_inside():
    """SampleWarp_Disc.cs:7-12 (forward half: points land in the unit disc)."""
    for u in [(0.1, 0.2), (0.9, 0.3), (0.5, 0.5), (0.0, 1.0)]:
        p = O.warp_disc(*u)
        assert np.hypot(*p) <= 1 + 1e-6


# ---- Background_EnvironmentMap.cs:8-157 ----
def env_scene(image):
    sc = Scene()
    m = quad_mesh()
    m.Material = DiffuseMaterial()
    sc.Meshes.append(m)
    sc.Background = EnvironmentMap(image)
    return O.OracleScene.from_scene(sc, commit=False)


def simple_map():
    img = RgbImage(512, 256)
    img.AtomicAdd(128, 64, RgbColor.White * 10)
    return env_scene(img)


def test_env_radiance_ten_and_zero():
    o = simple_map()
    assert np.all(o.env_radiance([0, 1, 1]) == 10)
    assert np.all(o.env_radiance([0, -1, 0]) == 0)
    assert np.all(o.env_radiance([-1, 0, 0]) == 0)


def test_env_rotation():
    img = RgbImage(512, 256)
    img.AtomicAdd(0, 128, RgbColor.White * 10)
    img.AtomicAdd(128, 128, RgbColor.White * 5)
    o = env_scene(img)
    assert np.all(o.env_radiance([1, 0, 0]) == 10)
    assert np.all(o.env_radiance([0, 0, 1]) == 5)


def test_env_sampling_pdf_and_estimator():
    """DirectionSampling_PdfShouldBeConsistent :72-80, _EstimatorShouldBeCorrect :82-95."""
    o = simple_map()
    d, pdf, w = o.env_sample(0.2, 0.2)
    p2 = o.env_pdf(d)
    assert eq(pdf, p2, 3)
    expected = o.env_radiance(d) / np.float32(p2)
    assert np.all(expected == w)


# ---- Scene_Assemble.cs:50-82 ----
def dummy_scene():
    sc = Scene()
    m0 = Mesh([[-1, 10, -1], [1, 10, -1], [1, 10, 1], [-1, 10, 1]], [0, 1, 2, 0, 2, 3])
    m0.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor(0, 0, 1))))
    m1 = Mesh([[-1, -10, -1], [1, -10, -1], [1, -10, 1], [-1, -10, 1]], [0, 1, 2, 0, 2, 3])
    m1.Material = GenericMaterial(GenericMaterial.Parameters(BaseColor=TextureRgb(RgbColor(1, 0, 0))))
    sc.Meshes += [m0, m1]
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, 0], [0, 5, 0], [0, 0, 1]), 90)
    sc.FrameBuffer = FrameBuffer(1, 1)
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(m0, RgbColor(1, 1, 1)))
    return sc


def test_scene_two_quads_intersection():
    sc = dummy_scene()
    o = O.OracleScene.from_scene(sc)
    org, d = o.camera_ray(0.5, 0.5)
    t, u, v, tri = o.trace(np.concatenate([org, [0], d, [np.inf]]).astype(np.float32))
    assert tri[0] >= 0
    assert eq(10.0, t[0], 4)


def test_scene_emitters_subdivided():
    sc = dummy_scene()
    o = O.OracleScene.from_scene(sc)
    assert o.num_emitters() == 2
    assert o.query_emitter(0, 0) == 0 and o.query_emitter(0, 1) == 1
    assert o.query_emitter(1, 0) == -1


def test_scene_invalid_without_material():
    sc = dummy_scene()
    sc.Meshes[0].Material = None
    assert not sc.IsValid


# ---- Emitter_Diffuse.cs:285-315 (one-sided emission) ----
def test_emitter_one_sided():
    sc = Scene()
    m = Mesh([[-1, 10, -1], [1, 10, -1], [1, 10, 1], [-1, 10, 1]], [0, 1, 2, 0, 2, 3], shadingNormals=[[0, 1, 0]] * 4)
    m.Material = DiffuseMaterial()
    sc.Meshes.append(m)
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(m, RgbColor.White))
    o = O.OracleScene.from_scene(sc, commit=False)
    pt = np.array([0, 10, 0, 0, -1, 0, 0, 1, 0, 0, 0], np.float32)
    assert o.emitter_radiance(0, pt, [0, 1, 1])[0] > 0
    assert o.emitter_radiance(0, pt, [0, -1, 1])[0] == 0


# ---- Mesh_Sampling.cs:9-125 (pdf of uniform area sampling over the mesh's emitters) ----
def test_triangle_area_pdf():
    sc = Scene()
    m = Mesh([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, -1], [0, 0, -1], [0, 0, 0]], [0, 1, 2, 3, 4, 5])
    m.Material = DiffuseMaterial()
    sc.Meshes.append(m)
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(m, RgbColor.White))
    o = O.OracleScene.from_scene(sc, commit=False)
    assert eq(1 / 2.0, o.emitter_sample(0, 0.3, 0.4)[9], 4)   # area 2
    assert eq(1 / 0.5, o.emitter_sample(1, 0.3, 0.4)[9], 4)   # area 0.5


def test_glossy_emitter_lobe():
    """GlossyEmitter.EmittedRadiance (GlossyEmitter.cs:36-40): radiance * cos^n * (n+1)/(2 pi)."""
    sc = Scene()
    m = Mesh([[-1, 10, -1], [1, 10, -1], [1, 10, 1], [-1, 10, 1]], [0, 1, 2, 0, 2, 3], shadingNormals=[[0, 1, 0]] * 4)
    m.Material = DiffuseMaterial()
    sc.Meshes.append(m)
    sc.Emitters.extend(GlossyEmitter.MakeFromMesh(m, RgbColor.White, 50))
    o = O.OracleScene.from_scene(sc, commit=False)
    pt = np.array([0, 10, 0, 0, -1, 0, 0, 1, 0, 0, 0], np.float32)
    d = norm([0, 1, 0.2])
    e = o.emitter_radiance(0, pt, d)
    expect = (d[1] ** 50) * 51 / (2 * math.pi)
    assert abs(e[0] - expect) <= 1e-5 * expect


# ---- RNG (Sampling/RNG.cs:90-118): restated independently in numpy ----
def _pcg(x):
    x = np.uint64(x)
    s = (x * np.uint64(747796405) + np.uint64(2891336453)) & np.uint64(0xFFFFFFFF)
    w = (((s >> ((s >> np.uint64(28)) + np.uint64(4))) ^ s) * np.uint64(277803737)) & np.uint64(0xFFFFFFFF)
    return int((w >> np.uint64(22)) ^ w)


def _fnv(h, d):
    for k in range(4):
        h = ((h * 16777619) & 0xFFFFFFFF) ^ ((d >> (8 * k)) & 0xFF)
    return h


def test_rng_hashseed_and_stream():
    for b, c, s in [(0xC030114, 0, 0), (571298512, 12345, 7), (1, 2**31 + 5, 511)]:
        h = _fnv(_fnv(_fnv(2166136261, _pcg(b)), _pcg(c)), _pcg(s))
        assert O.rng_hashseed(b, c, s) == _pcg(h)
    state = 0xDEADBEEF
    out = []
    for _ in range(16):
        w = ((((state >> ((state >> 28) + 4)) ^ state) * 277803737) & 0xFFFFFFFF)
        state = (state * 747796405 + 2891336453) & 0xFFFFFFFF
        out.append((w >> 22) ^ w)
    assert list(O.rng_stream(0xDEADBEEF, 16)) == out
    f = O.rng_floats(0xDEADBEEF, 16)
    assert np.all(f == (np.array(out, np.float64).astype(np.float32) / np.float32(4294967295.0)))


def test_rng_nextint_lemire():
    vals, _ = O.rng_ints(0x1234567, 50, 1000)
    assert vals.max() < 50
    assert len(set(vals.tolist())) == 50


# ---------------------------------------------------------------------------------------------
# The FP64 BVH query that referees the GPU's intersection parity on the benchmark scenes
# (tests/test_gpu_intersection.py) equals FP64 brute force: same closest triangle and distance, and
# the runner-up distance equals the nearest hit among all other triangles.
def test_oracle_bvh_two_hit_query_equals_brute_force():
    rng = np.random.default_rng(4)
    n = 400
    c = rng.uniform(-5, 5, size=(n, 1, 3))
    v = (c + rng.normal(scale=0.6, size=(n, 3, 3))).astype(np.float32)
    sc = Scene()
    m = Mesh(v.reshape(-1, 3), np.arange(3 * n, dtype=np.int32))
    m.Material = DiffuseMaterial()
    sc.Meshes.append(m)
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(m, RgbColor.White))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, 12], [0, 0, 0], [0, 1, 0]), 40)
    sc.FrameBuffer = FrameBuffer(8, 8)
    o = O.OracleScene.from_scene(sc, fp64=True)
    k = 1500
    org = rng.uniform(-8, 8, size=(k, 3))
    d = rng.uniform(-4, 4, size=(k, 3)) - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((k, 8), np.float32)
    rays[:, 0:3], rays[:, 4:7], rays[:, 7] = org, d, np.inf
    hits, second = o.trace_two64(rays)
    ref, ref2 = o.trace_brute64(rays[:, 0:3].astype(np.float64), rays[:, 4:7].astype(np.float64), with_second=True)
    assert np.array_equal(hits[:, 3], ref[:, 3])
    hit = ref[:, 3] >= 0
    assert hit.sum() > k // 4
    assert np.array_equal(hits[hit, 0], ref[hit, 0])
    assert np.array_equal(second[hit], ref2[hit])


# ---- Material_SampleTransform.cs:119-304: albedo by BSDF sampling against uniform-sphere sampling,
# and the pdf integrating to one, 1M samples each, 99% confidence intervals that must overlap ----
def _sampling_cases():
    white = TextureRgb(RgbColor(1, 1, 1))
    diffuse = lambda: DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=white, Transmitter=True))
    rough = lambda: GenericMaterial(GenericMaterial.Parameters(BaseColor=white, Roughness=TextureMono(0.9), IndexOfRefraction=1.1))
    glossy = lambda: GenericMaterial(GenericMaterial.Parameters(BaseColor=white, Roughness=TextureMono(0.2), Metallic=0.6))
    glass = lambda: GenericMaterial(GenericMaterial.Parameters(Roughness=TextureMono(0.1), Anisotropic=0.0, IndexOfRefraction=1.45, Metallic=0.0,
                                                               SpecularTintStrength=0.0, SpecularTransmittance=1.0))
    return [
        ("Diffuse_AlbedoShouldMatch", diffuse, (1, 0, 0.1), "albedo"),                              # :119-126
        ("Diffuse_PDFShouldBeDensity", diffuse, (1, 0, 0.1), "pdf"),                                # :128-135
        ("GenericRough_AlbedoShouldMatch", rough, (0, 0, 1), "albedo"),                             # :137-145
        ("GenericRough_PDFShouldBeDensity", rough, (0, 0, 1), "pdf"),                               # :147-155
        ("GenericGlossy_AlongNormal_AlbedoShouldMatch", glossy, (0, 0, 1), "albedo"),               # :157-165
        ("GenericGlossy_AlongNormal_PDFShouldBeDensity", glossy, (0, 0, 1), "pdf"),                 # :167-175
        ("GenericGlossy_AlongNormal_Underneath_AlbedoShouldMatch", glossy, (0, 0, -1), "albedo"),   # :177-185
        ("GenericGlossy_AlongNormal_Underneath_PDFShouldBeDensity", glossy, (0, 0, -1), "pdf"),     # :187-195
        ("GenericGlossy_GrazingAngle_AlbedoShouldMatch", glossy, (1, 0, 0.01), "albedo"),           # :197-205
        ("GenericGlossy_GrazingAngle_PDFShouldBeDensity", glossy, (1, 0, 0.01), "pdf"),             # :207-215
        ("GenericGlass_AlongNormal_AlbedoShouldMatch", glass, (0, 0, 1), "albedo"),                 # :217-228
        ("GenericGlass_GrazingAngle_AlbedoShouldMatch", glass, (1, 0, 0.01), "albedo"),             # :230-241
        ("GenericGlass_GrazingAngle_PDFShouldBeDensity", glass, (1, 0, 0.01), "pdf"),               # :243-254
        ("GenericGlass_GrazingAngle_Underneath_AlbedoShouldMatch", glass, (1, 0, -1.1), "albedo"),  # :256-267
        ("GenericGlass_GrazingAngle_Underneath_PDFShouldBeDensity", glass, (1, 0, -1.1), "pdf"),    # :269-280
    ]


SAMPLING_CASES = _sampling_cases()
# MakeDummyHit (:11-23): the quad at z = -2 hit from the origin straight down; face normal +z and no
# shading normals, so the shading normal is +z too.
SAMPLING_HIT = np.array([0, 0, -2, 0, 0, 1, 0, 0, 1, 0.25, 0.25], np.float32)


def overlap(a, b):
    """Material_SampleTransform.cs:94: two intervals overlap."""
    return b[0] < a[1] and b[1] > a[0]


@pytest.mark.parametrize("name,make,out,kind", SAMPLING_CASES, ids=[c[0] for c in SAMPLING_CASES])
def test_material_sample_transform(name, make, out, kind):
    o = material_scene(make())
    od = norm(out)
    if kind == "albedo":  # IntegrateBSDF :96-117
        uni = o.material_integrate(0, SAMPLING_HIT, od, 0)
        imp = o.material_integrate(0, SAMPLING_HIT, od, 1)
        assert overlap(uni, imp), (uni, imp)
    else:  # IntegratePdf :71-88
        ci = o.material_integrate(0, SAMPLING_HIT, od, 2)
        assert overlap(ci, (1.0, 1.0)), ci


@pytest.mark.parametrize("rough,ox,oy,oz", [(0.9, 1, 0, 0.1), (0.1, 1, 0, 0.1), (0.9, 1, 0, 1), (0.1, 1, 0, 1)])
def test_trowbridge_reitz_pdf_is_a_density(rough, ox, oy, oz):
    """TrowbridgeReitzDistribution_ShouldBeValidPDF :282-303."""
    a = max(0.001, np.float32(rough) * np.float32(rough))
    ci = O.ggx_pdf_integrate(a, a, norm((ox, oy, oz)))
    assert overlap(ci, (1.0, 1.0)), ci


# ---- Mesh_Attributes.cs:9-75: shading-normal interpolation and the CCW face-normal default ----
def _one_mesh_scene(mesh):
    sc = Scene()
    mesh.Material = DiffuseMaterial()
    sc.Meshes.append(mesh)
    return O.OracleScene.from_scene(sc, commit=False)


def test_mesh_shading_normals_should_be_set():
    """ShadingNormals_ShouldBeSet :9-47."""
    V = [[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, -1], [1, 0, -1], [-1, 0, 1]]
    N = [[1, 0, 0]] * 3 + [[1, 0, -1]] * 3
    o = _one_mesh_scene(Mesh(V, [0, 1, 2, 3, 4, 5], shadingNormals=N))
    n1, n2 = o.mesh_shading_normal(0, 0, 0.5, 0.5), o.mesh_shading_normal(0, 1, 0.5, 0.5)
    assert eq(n1[0], 1, 3) and eq(n1[1], 0, 3) and eq(n1[2], 0, 3)
    assert eq(n2[0], 1 / math.sqrt(2), 3) and eq(n2[1], 0, 3) and eq(n2[2], -1 / math.sqrt(2), 3)


def test_mesh_shading_normals_default_to_the_ccw_face_normal():
    """ShadingNormals_ShouldBeInitialized_CCW :49-74."""
    o = _one_mesh_scene(Mesh([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], [0, 1, 2, 0, 2, 3]))
    for uv in ((0.5, 0.25), (0.25, 0.5)):
        n = o.mesh_shading_normal(0, 0, *uv)
        assert eq(n[0], 0, 3) and eq(n[1], -1, 3) and eq(n[2], 0, 3)


# ---- Emitter_Diffuse.cs:205-233, Emitter_Glossy.cs:7-34: SampleRay inverted by SampleRayInverse ----
@pytest.mark.parametrize("glossy", [False, True], ids=["diffuse", "glossy"])
def test_emitted_rays_sample_inverse(glossy):
    m = Mesh([[-1, 10, -1], [1, 10, -1], [1, 10, 1], [-1, 10, 1]], [0, 1, 2, 0, 2, 3], shadingNormals=[[0, 1, 0]] * 4)
    m.Material = DiffuseMaterial()
    sc = Scene()
    sc.Meshes.append(m)
    sc.Emitters.extend(GlossyEmitter.MakeFromMesh(m, RgbColor.White, 50) if glossy else DiffuseEmitter.MakeFromMesh(m, RgbColor.White))
    o = O.OracleScene.from_scene(sc, commit=False)
    pos_p, dir_p, _, _, _, _ = o.emitter_ray_roundtrip(0, (0.3, 0.8), (0.56, 0.03))
    assert eq(pos_p[0], 0.3, 3) and eq(pos_p[1], 0.8, 3)
    assert eq(dir_p[0], 0.56, 3) and eq(dir_p[1], 0.03, 3)
