"""Frame-buffer layers computed in the GPU film fold: the error metrics against a reference image
after every iteration (FrameBuffer.cs:276-277, 378-383) and the VarianceLayer
(Images/VarianceLayer.cs:41-84)."""
import numpy as np
import pytest

from oracle import film_metrics as F
from oracle import pyoracle as O
from seesharp_gb300 import (DiffuseMaterial, EnvironmentMap, FrameBuffer, Matrix4x4, Mesh, PathTracer, PerspectiveCamera, Pixel, RgbColor,
                            RgbImage, Scene, TextureRgb, workloads)

pytestmark = pytest.mark.gpu

W, H = 64, 48


def _render(sc, spp, seed=0xC030114):
    sc.FrameBuffer.Reset()
    pt = PathTracer(TotalSpp=spp, MaxDepth=5, BaseSeed=seed)
    pt.Render(sc)
    return sc.FrameBuffer.Image.data.copy()


def test_error_metrics_equal_the_metrics_of_each_iterations_film():
    """The film after iteration k equals a k-spp render (the running mean is wave-independent), so
    the per-iteration MSE / RelMSE must equal the metrics of those films."""
    sc = workloads.cornell_box(W, H)
    sc.Prepare()
    ref = _render(sc, 256, seed=77)
    S = 6
    fb = FrameBuffer(W, H)
    fb.ReferenceImage = RgbImage(ref)
    sc.FrameBuffer = fb
    PathTracer(TotalSpp=S, MaxDepth=5).Render(sc)
    layered = fb.Image.data.copy()
    errs = fb.Errors
    assert len(errs) == S
    sc.FrameBuffer = FrameBuffer(W, H)
    assert np.array_equal(layered, _render(sc, S))
    r64 = ref.astype(np.float64)
    for k in range(1, S + 1):
        film = _render(sc, k)
        d = (film - ref).astype(np.float64)
        mse, rel = np.mean(d * d), np.mean(d * d / (r64 * r64 + 0.01))
        assert errs[k - 1][1] == pytest.approx(mse, rel=1e-9) and errs[k - 1][2] == pytest.approx(rel, rel=1e-9)
        # the outlier-rejecting RelMSE: 3072 pixels, the largest 3 errors dropped
        assert errs[k - 1][3] == pytest.approx(F.relmse_outlier_rejection(film, ref), rel=1e-9)
        assert errs[k - 1][3] <= errs[k - 1][2] * (1 + 1e-9)
    assert errs[-1][2] < errs[0][2]


@pytest.mark.parametrize("w,h", [(100, 80), (31, 17)])
def test_outlier_rejecting_relmse_drops_the_fireflies(w, h):
    """8000 pixels drop 8: a reference that is black at the 8 brightest pixels (the light) makes
    those pixels' errors dominate the plain RelMSE, and the rejection removes them.  527 pixels
    drop none (the plain RelMSE)."""
    sc = workloads.cornell_box(w, h)
    sc.Prepare()
    ref = _render(sc, 64, seed=5)
    bad = ref.copy()
    if w * h >= 1000:
        flat = bad.reshape(-1, 3)
        flat[np.argsort(-ref.reshape(-1, 3).mean(axis=1))[:8]] = 0.0
    fb = FrameBuffer(w, h)
    fb.ReferenceImage = RgbImage(bad)
    sc.FrameBuffer = fb
    PathTracer(TotalSpp=2, MaxDepth=5).Render(sc)
    film = fb.Image.data
    got = fb.Errors[-1][3]
    assert got == pytest.approx(F.relmse_outlier_rejection(film, bad), rel=1e-9)
    if w * h >= 1000:
        assert got < 0.5 * fb.Errors[-1][2]
    else:
        assert got == pytest.approx(fb.Errors[-1][2], rel=1e-6)


def test_variance_layer_matches_the_oracle():
    """The variance image from the oracle's per-iteration path values (the same running means in
    FP32, the 3x3 box, the relative variance); pixels whose paths differ by an FP32 decision flip
    are allowed to disagree."""
    S = 8
    sc = workloads.cornell_box(W, H)
    sc.FrameBuffer = FrameBuffer(W, H, flags=FrameBuffer.Flags.Recommended | FrameBuffer.Flags.EstimatePixelVariance)
    sc.Prepare()
    PathTracer(TotalSpp=S, MaxDepth=5).Render(sc)
    var = sc.FrameBuffer.PixelVariance.Image.data[:, :, 0]
    avg = sc.FrameBuffer.PixelVariance.Average
    o = O.OracleScene.from_scene(sc)
    p = o.params(W, H, S, 5)
    pix = np.arange(W * H, dtype=np.int32)
    mean = np.zeros(W * H, np.float32)
    moment = np.zeros(W * H, np.float32)
    for it in range(S):
        rgb, _, _ = o.render_paths(p, it, pix)
        val = (rgb[:, 0] + rgb[:, 1] + rgb[:, 2]) / np.float32(3)
        val = np.where(np.isfinite(val), val, np.float32(0)).astype(np.float32)
        k = np.float32(it + 1)
        if it > 0:
            mean = mean * ((k - 1) / k)
            moment = moment * ((k - 1) / k)
        moment = moment + val * val / k
        mean = mean + val / k
    m2, o2 = mean.reshape(H, W).astype(np.float64), moment.reshape(H, W).astype(np.float64)
    pad_m, pad_o = np.pad(m2, 1), np.pad(o2, 1)
    cnt = np.pad(np.ones((H, W)), 1)
    box = lambda a: sum(a[1 + dy:1 + dy + H, 1 + dx:1 + dx + W] for dy in (-1, 0, 1) for dx in (-1, 0, 1))
    bm, bo = box(pad_m) / box(cnt), box(pad_o) / box(cnt)
    want = (bo - bm * bm) / (bm * bm + 0.001)
    ok = np.abs(var - want) <= 1e-3 + 1e-3 * np.abs(want)
    assert ok.mean() >= 0.95, ok.mean()
    assert avg == pytest.approx(want.mean(), rel=0.02)
    assert np.isfinite(var).all() and avg > 0


def test_denoiser_feature_layers_match_the_primary_hits():
    """The "albedo" and "normal" layers (DenoiseBuffers.LogPrimaryHit, PathTracer.cs:336-339):
    running means over the iterations of the primary hit's base colour and shading normal, here
    rebuilt from the oracle's camera rays (the same jitter from RNG(BaseSeed, pixel, iteration)) and
    its intersector; the Cornell box has constant colours and no vertex normals."""
    S = 5
    w, h = 40, 30
    sc = workloads.cornell_box(w, h)
    sc.Prepare()
    sc.FrameBuffer.Reset()
    PathTracer(TotalSpp=S, MaxDepth=3).Render(sc)
    alb = sc.FrameBuffer.GetLayer("albedo").Image.data
    nrm = sc.FrameBuffer.GetLayer("normal").Image.data
    o = O.OracleScene.from_scene(sc)
    # global triangle -> (base colour, face normal)
    cols, norms = [], []
    for m in sc.Meshes:
        V, I = m.Vertices, m.Indices.reshape(-1, 3)
        c = m.Material.MaterialParameters.BaseColor.constColor.array()
        for f in I:
            n = np.cross(V[f[1]] - V[f[0]], V[f[2]] - V[f[0]]).astype(np.float32)
            norms.append(n / np.float32(np.sqrt(np.dot(n, n))))
            cols.append(c)
    cols, norms = np.array(cols, np.float32), np.array(norms, np.float32)
    want_a = np.zeros((h, w, 3), np.float32)
    want_n = np.zeros((h, w, 3), np.float32)
    for it in range(S):
        rays = np.zeros((w * h, 8), np.float32)
        for pix in range(w * h):
            u2 = O.rng_floats(O.rng_hashseed(0xC030114, pix, it), 2)
            org, d = o.camera_ray(np.float32(pix % w) + u2[0], np.float32(pix // w) + u2[1])
            rays[pix, 0:3], rays[pix, 4:7], rays[pix, 7] = org, d, np.inf
        _, _, _, tri = o.trace(rays)
        a = np.where(tri[:, None] >= 0, cols[np.maximum(tri, 0)], 0).reshape(h, w, 3).astype(np.float32)
        n = np.where(tri[:, None] >= 0, norms[np.maximum(tri, 0)], 0).reshape(h, w, 3).astype(np.float32)
        k = np.float32(it + 1)
        if it > 0:
            want_a = want_a * ((k - 1) / k)
            want_n = want_n * ((k - 1) / k)
        want_a = want_a + a / k
        want_n = want_n + n / k
    ok_a = np.all(np.abs(alb - want_a) <= 1e-5, axis=2).mean()
    ok_n = np.all(np.abs(nrm - want_n) <= 1e-5, axis=2).mean()
    assert ok_a >= 0.99 and ok_n >= 0.99, (ok_a, ok_n)


def test_layers_resume_like_the_film():
    """Rendering 3 + 4 iterations equals rendering 7: film, variance layer, feature layers and the
    outlier replay cache."""
    def run(steps):
        sc = workloads.cornell_box(W, H)
        sc.FrameBuffer = FrameBuffer(W, H, flags=FrameBuffer.Flags.Recommended | FrameBuffer.Flags.EstimatePixelVariance)
        sc.Prepare()
        for s in steps:
            PathTracer(TotalSpp=s, MaxDepth=4).Render(sc)
        fb = sc.FrameBuffer
        return (fb.Image.data.copy(), fb.PixelVariance.Image.data.copy(), fb.PixelVariance.Average, fb.GetLayer("albedo").Image.data.copy(),
                fb.OutlierCache.weight.copy(), fb.OutlierCache.iteration.copy())
    a, b = run([7]), run([3, 7])
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2] and np.array_equal(a[3], b[3])
    assert np.array_equal(a[4], b[4]) and np.array_equal(a[5], b[5])


def test_outlier_cache_matches_the_oracle():
    """OutlierReplayCache (OutlierReplayCache.cs:9-35): per pixel the 4 samples of largest channel
    average, in the .NET heap's array order, against the oracle's restatement fed with the oracle's
    per-iteration path values.  Pixels whose paths differ by an FP32 decision flip may disagree."""
    S, w, h = 9, 40, 30
    sc = workloads.cornell_box(w, h)
    sc.Prepare()
    sc.FrameBuffer.Reset()
    PathTracer(TotalSpp=S, MaxDepth=5).Render(sc)
    oc = sc.FrameBuffer.OutlierCache
    o = O.OracleScene.from_scene(sc)
    p = o.params(w, h, S, 5)
    pix = np.arange(w * h, dtype=np.int32)
    vals = np.stack([o.render_paths(p, it, pix)[0].reshape(h, w, 3) for it in range(S)])
    ow, oi = F.outlier_cache(vals, 4)
    same = np.all(oc.iteration == oi, axis=2) & np.all(np.abs(oc.weight - ow) <= 1e-4 * np.abs(ow) + 1e-6, axis=2)
    assert same.mean() >= 0.97, same.mean()
    assert (oc.iteration >= 0).all()  # 9 finite samples fill every heap
    # the strongest sample of a pixel, looked up as OutlierCacheTest.cs:27-36 does
    y, x = np.argwhere(same)[len(np.argwhere(same)) // 2]
    q = oc.GetPixelOutlier(Pixel(int(x), int(y)))
    best = max(q.UnorderedItems, key=lambda i: i.Priority)
    assert q.Count == 4 and best.Element.Iteration == oi[y, x][np.argmax(ow[y, x])]


def test_replay_pixel_reproduces_the_cached_outliers():
    """PathTracer.ReplayPixel (PathTracer.cs:60-68) re-renders one (pixel, iteration) path from its
    seed: its channel average equals the outlier cache's priority for that entry bit for bit, as
    OutlierCacheTest.cs:24-38 relies on, and iteration 0 equals the 1-spp film."""
    S, w, h = 6, 24, 16
    sc = workloads.cornell_box(w, h)
    sc.Prepare()
    pt = PathTracer(TotalSpp=S, MaxDepth=5)
    pt.Render(sc)
    oc = sc.FrameBuffer.OutlierCache
    rng = np.random.default_rng(4)
    for col, row in zip(rng.integers(0, w, 12), rng.integers(0, h, 12)):
        q = oc.GetPixelOutlier(Pixel(int(col), int(row)))
        for item in q.UnorderedItems:
            graph, est = pt.ReplayPixel(sc, Pixel(int(col), int(row)), item.Element.Iteration)
            r, g, b = (np.float32(x) for x in est.array())
            assert graph is None and np.float32((r + g + b) / np.float32(3)) == np.float32(item.Priority)
    # a batch of paths through the C ABI: iteration 0 of every pixel is the 1-spp film
    sc.FrameBuffer = FrameBuffer(w, h)
    PathTracer(TotalSpp=1, MaxDepth=5).Render(sc)
    film = sc.FrameBuffer.Image.data.reshape(-1, 3)
    rgb, _ = sc.native.render_paths(pt.params(sc), np.arange(w * h), np.zeros(w * h))
    assert np.array_equal(rgb, film)


def _constant_background_scene(w, h):
    sc = Scene()
    tri = Mesh([[-1, -1, 5], [1, -1, 5], [0, 1, 5]], [0, 1, 2])  # behind the camera
    tri.Material = DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor(0.5, 0.5, 0.5))))
    sc.Meshes.append(tri)
    sc.Background = EnvironmentMap(RgbImage(np.tile(np.array([0.5, 0.25, 1.0], np.float32), (4, 8, 1))))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, 0], [0, 0, -1], [0, 1, 0]), 50)
    sc.FrameBuffer = FrameBuffer(w, h)
    return sc


@pytest.mark.parametrize("n", [0, 1, 4, 8])
def test_outlier_cache_ties(n):
    """Every camera ray escapes into a constant background, so every sample of every pixel has the
    same value: the heap keeps the first n iterations in order (equal samples neither sift nor
    replace the root)."""
    S = 6
    sc = _constant_background_scene(16, 12)
    sc.FrameBuffer.NumOutliersToTrack = n
    sc.Prepare()
    PathTracer(TotalSpp=S, MaxDepth=3).Render(sc)
    oc = sc.FrameBuffer.OutlierCache
    assert np.allclose(sc.FrameBuffer.Image.data, np.array([0.5, 0.25, 1.0], np.float32), rtol=1e-6, atol=0)
    want = [i if i < S else -1 for i in range(n)]
    assert oc.iteration.shape == (12, 16, n) and np.all(oc.iteration == np.array(want, np.int32))
    kept = oc.iteration >= 0
    assert np.all(oc.weight[kept] == np.float32((np.float32(0.5) + np.float32(0.25) + np.float32(1.0)) / np.float32(3)))
