"""Path-replay adjoint (sst_forward / sst_backward) on the differentiation workload: the Cornell
box with a textured GenericMaterial back wall, a GenericMaterial roughness per box and the
ceiling light's RGB radiance, L2 loss to a target rendered with perturbed parameters.

* FP64 replay: the oracle re-renders every path of the same seeds in double precision and
  differentiates each BSDF by central differences (h = 1e-6).  The GPU gradients (FP32, dual
  numbers) agree to 2% relative L2 in every parameter group.
* Central finite differences with common random numbers (h = 1e-3, same seeds at theta +- h) on
  200 seeded entries.  The sampled paths do not depend on texels or on the emitter's radiance
  (the back wall has no metallic or tinted specular part, and at depth 5 Russian roulette cannot
  end a path before the depth limit does), so the estimator is smooth in those entries and the
  adjoint equals its derivative up to FP32 rounding: 2% relative L2.  Box roughness moves the
  sampled directions; the detached-sampling adjoint and the finite difference then agree in
  expectation only, which a separate, converged comparison checks to 15%.
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from seesharp_gb300 import PathTracer, RgbColor, workloads
from seesharp_gb300.adjoint import DifferentiableRender, l2_loss

pytestmark = pytest.mark.gpu

ROUGH0, RAD0 = (0.3, 0.6), (17.0, 12.0, 4.0)


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def setup(width, height, spp, tex_res, seed=11):
    sc, tex, boxes, lights = workloads.cornell_box_differentiable(width, height, tex_res=tex_res, roughness=ROUGH0, radiance=RAD0)
    sc.Prepare()
    pt = PathTracer(TotalSpp=spp, MaxDepth=5)
    dr = DifferentiableRender(sc, pt, texture=tex, roughness_materials=boxes, emitters=[lights])
    # target: the same scene with seeded perturbed parameters and another seed
    rng = np.random.default_rng(seed)
    tex0 = tex.Image.data.copy()
    t_tex = np.clip(tex0 * (1 + 0.3 * rng.standard_normal(tex0.shape)), 0.02, 0.98).astype(np.float32)
    t_rough = np.asarray(ROUGH0) + [0.15, -0.2]
    t_rad = np.asarray(RAD0) * [0.8, 1.1, 1.3]
    dr.params.baseSeed = 0x5EED
    target = dr.forward(t_tex, t_rough, t_rad)
    dr.params.baseSeed = pt.BaseSeed
    image = dr.forward(tex0, ROUGH0, RAD0)
    return sc, dr, tex0, image, target


def test_adjoint_matches_fp64_replay():
    sc, dr, tex0, image, target = setup(64, 64, 8, 32)
    loss, dldi = l2_loss(image, target)
    g = dr.backward(dldi)
    o = O.OracleScene.from_scene(sc, fp64=True)
    P = o.params(64, 64, 8, 5, baseSeed=dr.params.baseSeed)
    ref = o.adjoint(P, dldi, dr.n_tex, dr.n_mat, dr.n_em)
    raw = g["raw"]
    for key in ("textures", "materialBaseColor", "materialRoughness", "emitterRadiance"):
        assert np.all(np.isfinite(raw[key])), key
        if np.linalg.norm(ref[key]) > 0:
            assert rel_l2(raw[key], ref[key]) <= 0.02, (key, rel_l2(raw[key], ref[key]))
    # every parameter group receives gradient
    assert np.linalg.norm(g["texture"]) > 0 and np.all(g["roughness"] != 0) and np.all(g["radiance"] != 0)


def test_adjoint_matches_fp64_replay_at_the_differentiation_size():
    """The differentiation configuration itself (512 x 512, 32 spp, depth 5, 256 x 256 texture)
    against the FP64 replay, on every 64th pixel: dLoss/dImage is the L2 loss gradient there and
    zero elsewhere, so the replay covers 4096 pixels x 32 paths."""
    sc, dr, tex0, image, target = setup(512, 512, 32, 256)
    loss, dldi = l2_loss(image, target)
    mask = np.zeros(512 * 512, bool)
    mask[::64] = True
    dldi = np.where(mask.reshape(512, 512, 1), dldi, 0).astype(np.float32)
    g = dr.backward(dldi)["raw"]
    o = O.OracleScene.from_scene(sc, fp64=True)
    ref = o.adjoint(o.params(512, 512, 32, 5, baseSeed=dr.params.baseSeed), dldi, dr.n_tex, dr.n_mat, dr.n_em)
    for key in ("textures", "materialBaseColor", "materialRoughness", "emitterRadiance"):
        assert np.all(np.isfinite(g[key])), key
        if np.linalg.norm(ref[key]) > 0:
            assert rel_l2(g[key], ref[key]) <= 0.02, (key, rel_l2(g[key], ref[key]))
    assert np.count_nonzero(ref["textures"]) > 1000


def test_adjoint_large_combined_shape_matches_fp64_replay():
    """The large combined job's gradient shape at a reduced size: a 1024 x 1024 x 3 base-colour
    texture on the terrain and the roughness of every icosphere (60 here, 2000 in the full job),
    depth 10, against the FP64 replay of the same paths.  The texture gradient is compared in 4 x 4
    texel blocks: a hit's texel is floor(uv * 1024), and the FP32 and FP64 interpolations of uv
    differ by about 1e-7, which puts about 2e-4 of the lookups on the other side of a texel edge;
    those paths credit the neighbouring texel, which a block sum absorbs."""
    sc, tex, mats, cams = workloads.large_combined(96, 54, num_spheres=60, terrain_quads=64, tex_res=1024, num_lights=40, views=1)
    sc.Prepare()
    pt = PathTracer(TotalSpp=4, MaxDepth=10)
    dr = DifferentiableRender(sc, pt, texture=tex, roughness_materials=mats)
    rng = np.random.default_rng(8)
    tex0 = tex.Image.data.copy()
    r0 = np.array([m.MaterialParameters.Roughness.constColor for m in mats], np.float64)
    dr.params.baseSeed = 0x5EED
    target = dr.forward(np.clip(tex0 * (1 + 0.3 * rng.standard_normal(tex0.shape)), 0.02, 0.98).astype(np.float32),
                        np.clip(r0 + 0.2 * rng.standard_normal(r0.shape), 0.05, 1.0), None)
    dr.params.baseSeed = pt.BaseSeed
    image = dr.forward(tex0, r0, None)
    loss, dldi = l2_loss(image, target)
    g = dr.backward(dldi)
    o = O.OracleScene.from_scene(sc, fp64=True)
    ref = o.adjoint(o.params(96, 54, 4, 10, baseSeed=dr.params.baseSeed), dldi, dr.n_tex, dr.n_mat, dr.n_em)
    raw = g["raw"]

    def blocks(t):
        t = np.asarray(t, np.float64)[dr.tex_offset:dr.tex_offset + 1024 * 1024 * 3].reshape(256, 4, 256, 4, 3)
        return t.sum(axis=(1, 3))

    for key in ("textures", "materialRoughness"):
        assert np.all(np.isfinite(raw[key])), key
        assert np.linalg.norm(ref[key]) > 0, key
    assert rel_l2(blocks(raw["textures"]), blocks(ref["textures"])) <= 0.02, rel_l2(blocks(raw["textures"]), blocks(ref["textures"]))
    assert rel_l2(raw["materialRoughness"], ref["materialRoughness"]) <= 0.02, rel_l2(raw["materialRoughness"], ref["materialRoughness"])
    assert np.count_nonzero(g["roughness"]) >= 30 and g["texture"].shape == (1024, 1024, 3)


def _fd(dr, loss_of, theta, h):
    return (loss_of(theta + h) - loss_of(theta - h)) / (2 * h)


def test_adjoint_matches_central_differences():
    """200 seeded entries at the full differentiation size (512x512, 32 spp, depth 5, 256x256
    texture): 197 (texel, channel) entries and the 3 radiance channels."""
    sc, dr, tex0, image, target = setup(512, 512, 32, 256)
    loss, dldi = l2_loss(image, target)
    g = dr.backward(dldi)
    h = 1e-3
    rng = np.random.default_rng(2024)
    ent = rng.choice(tex0.size, size=197, replace=False)
    fd_tex, ad_tex = [], []
    t = tex0.copy().reshape(-1)
    for e in ent:
        base = float(t[e])

        def L(v):
            t[e] = v
            return l2_loss(dr.forward(t.reshape(tex0.shape), None, None), target)[0]

        fd_tex.append(_fd(dr, L, base, h))
        t[e] = base
        ad_tex.append(float(g["texture"].reshape(-1)[e]))
    dr.set_parameters(texture=tex0)
    fd_rad, ad_rad = [], []
    for c in range(3):
        def L(v, c=c):
            r = np.asarray(RAD0, np.float64).copy()
            r[c] = v
            return l2_loss(dr.forward(None, None, r), target)[0]

        fd_rad.append(_fd(dr, L, RAD0[c], h))
        ad_rad.append(float(g["radiance"][0, c]))
    dr.set_parameters(radiance=RAD0)
    assert np.count_nonzero(fd_tex) > 150
    assert rel_l2(ad_tex, fd_tex) <= 0.02, rel_l2(ad_tex, fd_tex)
    assert rel_l2(ad_rad, fd_rad) <= 0.02, (ad_rad, fd_rad)


def test_roughness_gradient_matches_central_differences_in_expectation():
    """Roughness moves the sampled directions, so the estimator jumps where a sampled ray changes
    what it hits: the variance of a central difference grows like 1/h.  With h = 0.05, 8192 spp
    and common random numbers the difference is converged to a few percent; the adjoint (detached
    sampling, an unbiased estimate of the same derivative) must agree to 15%."""
    W = H = 128
    sc, tex, boxes, lights = workloads.cornell_box_differentiable(W, H, tex_res=64, roughness=ROUGH0, radiance=RAD0)
    sc.Prepare()
    dr = DifferentiableRender(sc, PathTracer(TotalSpp=8192, MaxDepth=5), texture=tex, roughness_materials=boxes, emitters=[lights])
    w = (np.random.default_rng(0).standard_normal((H, W, 3)) ** 2).astype(np.float32)  # J = sum(w * image)
    dr.forward(None, ROUGH0, None)
    g = dr.backward(w)
    h = 0.05
    for k in range(2):
        r = np.asarray(ROUGH0, np.float64).copy()
        r[k] += h
        jp = float(np.sum(w * dr.forward(None, r, None)))
        r[k] -= 2 * h
        jm = float(np.sum(w * dr.forward(None, r, None)))
        fd = (jp - jm) / (2 * h)
        assert abs(g["roughness"][k] - fd) <= 0.15 * abs(fd), (k, g["roughness"][k], fd)
    dr.set_parameters(roughness=ROUGH0)
    # the boxes' constant base colour: tinted, metallic specular, so the colour channels couple and
    # the lobe-selection probabilities move with it (the same statistical comparison)
    mat, mid = boxes[1], dr.mat_ids[1]
    base0 = mat.MaterialParameters.BaseColor.constColor.array().copy()
    for c in range(3):
        js = []
        for sgn in (1, -1):
            b = base0.astype(np.float64).copy()
            b[c] += sgn * h
            mat.MaterialParameters.BaseColor.constColor = RgbColor(*b)
            sc.native.update_generic(mid, mat.MaterialParameters)
            js.append(float(np.sum(w * dr.forward())))
        fd = (js[0] - js[1]) / (2 * h)
        ad = g["raw"]["materialBaseColor"][mid, c]
        assert abs(ad - fd) <= 0.15 * abs(fd), (c, ad, fd)
    mat.MaterialParameters.BaseColor.constColor = RgbColor(*base0)
    sc.native.update_generic(mid, mat.MaterialParameters)


def test_backward_is_deterministic_and_linear_in_dldi():
    sc, dr, tex0, image, target = setup(48, 40, 4, 16)
    rng = np.random.default_rng(5)
    d1 = rng.standard_normal(image.shape).astype(np.float32)
    d2 = rng.standard_normal(image.shape).astype(np.float32)
    g1 = dr.backward(d1)["raw"]
    g2 = dr.backward(d2)["raw"]
    g12 = dr.backward((d1 + 2 * d2).astype(np.float32))["raw"]
    g1b = dr.backward(d1)["raw"]
    for k in g1:
        assert rel_l2(g1b[k], g1[k]) <= 1e-5
        if np.linalg.norm(g12[k]) > 0:
            assert rel_l2(g12[k], g1[k] + 2 * g2[k]) <= 1e-4


def test_forward_equals_render():
    sc, dr, tex0, image, target = setup(40, 48, 4, 16)
    sc.FrameBuffer.Reset()
    pt = PathTracer(TotalSpp=4, MaxDepth=5)
    pt.Render(sc)
    assert np.array_equal(sc.FrameBuffer.Image.data, image)


def test_batched_views_adjoint_equals_single_views():
    """sst_forward_batch / sst_backward_batch over two camera views of one scene: the images
    equal single-view forwards, the gradients the sum of the single-view gradients."""
    from seesharp_gb300 import Matrix4x4, PerspectiveCamera
    views = [(Matrix4x4.CreateLookAt([0, 0, 3.7], [0, 0, 0], [0, 1, 0]), 40.0),
             (Matrix4x4.CreateLookAt([0.4, 0.2, 3.2], [0, -0.1, 0], [0, 1, 0]), 50.0)]
    rng = np.random.default_rng(3)
    dl = [rng.standard_normal((40, 48, 3)).astype(np.float32) for _ in views]
    singles = []
    for (m, f), d in zip(views, dl):
        sc, tex, boxes, lights = workloads.cornell_box_differentiable(48, 40, tex_res=16)
        sc.Camera = PerspectiveCamera(m, f)
        sc.Prepare()
        dr = DifferentiableRender(sc, PathTracer(TotalSpp=4, MaxDepth=5), texture=tex, roughness_materials=boxes, emitters=[lights])
        img = dr.forward()
        singles.append((img, dr.backward(d)["raw"]))
    sc, tex, boxes, lights = workloads.cornell_box_differentiable(48, 40, tex_res=16)
    sc.Prepare()
    dr = DifferentiableRender(sc, PathTracer(TotalSpp=4, MaxDepth=5), texture=tex, roughness_materials=boxes, emitters=[lights], views=views)
    imgs = dr.forward()
    g = dr.backward(dl)["raw"]
    for img, (s_img, _) in zip(imgs, singles):
        assert np.array_equal(img, s_img)
    for k in g:
        ref = singles[0][1][k] + singles[1][1][k]
        if np.linalg.norm(ref) > 0:
            assert rel_l2(g[k], ref) <= 1e-4, (k, rel_l2(g[k], ref))
