"""Render statistics and limits through the C ABI: the frame buffer's NaN / Inf log
(SeeSharp.Tests/Core/FrameBuffer.cs:8-56, Images/FrameBuffer.cs:166-191), ShadingStats
(Shading/ShadingStats.cs, written by PathTracer.cs:256) against the oracle's count of the
reference's material calls, and MaximumRenderTimeMs (PathTracer.cs:219-227)."""
import json
import math
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from seesharp_gb300 import (DiffuseEmitter, DiffuseMaterial, FrameBuffer, Mesh, PathTracer, RgbColor, TextureRgb, _native, workloads)
from seesharp_gb300.workloads import _quad

pytestmark = pytest.mark.gpu


def nan_scene(w, h, flags=None):
    """The Cornell box with a small floor emitter whose radiance has a NaN channel: every path that
    hits it, or connects to it by next-event estimation, estimates a non-finite radiance."""
    sc = workloads.cornell_box(w, h)
    v, i = _quad([-0.9, -0.999, 0.9], [0.2, 0, 0], [0, 0, -0.2])  # normal +y
    q = Mesh(v, i)
    q.Material = DiffuseMaterial(DiffuseMaterial.Parameters(BaseColor=TextureRgb(RgbColor.Black)))
    sc.Meshes.append(q)
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(q, RgbColor(float("nan"), 1.0, 1.0)))
    sc.FrameBuffer = FrameBuffer(w, h, flags=flags)
    return sc


def _replay(sc, pt, pixels, iterations):
    p = pt.params(sc)
    return sc.native.render_paths(p, np.asarray(pixels, np.int32), np.asarray(iterations, np.int32))[0]


def test_nan_and_inf_are_logged_and_ignored(tmp_path):
    """FrameBuffer.cs:166-191: every non-finite estimate is counted; with IgnoreNanAndInf (the
    default, Flags.Recommended) it does not enter the film.  The log lists the first estimates in
    (iteration, pixel) order with the 1-based iteration, and each logged path replays to a
    non-finite estimate (NaNShouldBeLogged); the JSON metadata carries the same entries
    (NaNShouldBeLoggedInJson)."""
    W, H, S = 40, 32, 3
    sc = nan_scene(W, H)
    sc.FrameBuffer.filename = str(tmp_path / "nantest.exr")
    sc.Prepare()
    pt = PathTracer(TotalSpp=S, MaxDepth=3, EnableDenoiser=False)
    pt.Render(sc)
    st = pt.last_stats
    film = sc.FrameBuffer.Image.data
    assert np.isfinite(film).all()
    # every path of the render, replayed from its seed
    pix = np.tile(np.arange(W * H), S)
    its = np.repeat(np.arange(S), W * H)
    est = _replay(sc, pt, pix, its)
    bad = ~np.isfinite(est.mean(axis=1))
    assert bad.sum() > 4
    assert int(st.numNanOrInf) == int(bad.sum())
    # the log: the four smallest (iteration, pixel) keys, 1-based iterations
    keys = sorted(zip(its[bad] + 1, pix[bad]))[:4]
    warn = sc.FrameBuffer.NaNWarnings
    assert [(it, r * W + c) for (c, r, it) in warn] == [(int(a), int(b)) for a, b in keys]
    sc.FrameBuffer.WriteToFile()
    meta = json.load(open(str(tmp_path / "nantest.json")))
    assert [(w["Iteration"], w["Pixel"]["Col"], w["Pixel"]["Row"]) for w in meta["NaNWarnings"]] == [(it, c, r) for (c, r, it) in warn]


def test_nan_enters_the_film_without_the_ignore_flag():
    W, H, S = 32, 32, 2
    sc = nan_scene(W, H, flags=FrameBuffer.Flags.None_)
    sc.Prepare()
    pt = PathTracer(TotalSpp=S, MaxDepth=3, EnableDenoiser=False)
    pt.Render(sc)
    film = sc.FrameBuffer.Image.data
    est = _replay(sc, pt, np.tile(np.arange(W * H), S), np.repeat(np.arange(S), W * H)).reshape(S, H, W, 3)
    bad_pixels = (~np.isfinite(est.mean(axis=3))).any(axis=0)
    assert np.array_equal(~np.isfinite(film.mean(axis=2)), bad_pixels)
    assert int(pt.last_stats.numNanOrInf) == int((~np.isfinite(est.mean(axis=3))).sum())


@pytest.mark.parametrize("scene", ["cornell", "sphere_field", "environment"])
def test_shading_stats_equal_the_reference_counts(scene):
    """ShadingStats at 1 spp equal the oracle's count of the reference's material calls: a sample per
    sampled direction (plus an evaluation and a pdf for a DiffuseMaterial), and an evaluation and a
    pdf per next-event sample whose shadow ray is unoccluded.  FP32 decision flips between the two
    renders change a few paths, so the counts are compared to a relative 1e-3 (2e-3 with GenericMaterials)."""
    if scene == "cornell":
        sc, spp, depth, tol = workloads.cornell_box(64, 64), 1, 5, 1e-3
    elif scene == "sphere_field":
        sc, spp, depth, tol = workloads.sphere_field(12, 48, 48, level=3), 1, 8, 2e-3
    else:
        sc, spp, depth, tol = workloads.env_lit_box(48, 48), 2, 5, 2e-3
    sc.Prepare()
    pt = PathTracer(TotalSpp=spp, MaxDepth=depth, EnableDenoiser=False, CountShadingStats=True)
    pt.Render(sc)
    g = sc.FrameBuffer.MetaData["ShadingStats"]
    film_counted = sc.FrameBuffer.Image.data.copy()
    o = O.OracleScene.from_scene(sc)
    o.render(o.params(sc.FrameBuffer.Width, sc.FrameBuffer.Height, spp, depth))
    r = o.last_shading_stats
    assert r["NumMaterialSample"] > 0 and r["NumMaterialEval"] > r["NumMaterialSample"] // 2
    for k in ("NumMaterialEval", "NumMaterialSample", "NumMaterialPdf"):
        assert abs(g[k] - r[k]) <= tol * r[k], (k, g[k], r[k])
    # counting traces extra shadow rays but leaves the image unchanged
    sc.FrameBuffer.Reset()
    pt2 = PathTracer(TotalSpp=spp, MaxDepth=depth, EnableDenoiser=False)
    pt2.Render(sc)
    assert np.array_equal(sc.FrameBuffer.Image.data, film_counted)
    assert "ShadingStats" not in sc.FrameBuffer.MetaData or sc.FrameBuffer.MetaData["ShadingStats"] == g
    assert pt2.last_stats.numMaterialSample == 0


def test_maximum_render_time_stops_at_a_whole_iteration():
    """PathTracer.cs:219-227: before each iteration the render stops if the time so far plus the
    cost of one iteration would exceed MaximumRenderTimeMs.  The film is then the running mean of
    exactly the iterations rendered (bitwise the film of a render with that TotalSpp), and
    MetaData["NumIterations"] counts them."""
    sc = workloads.sphere_field(30, 256, 256, level=3)
    sc.Prepare()
    pt = PathTracer(TotalSpp=100000, MaxDepth=6, EnableDenoiser=False, MaximumRenderTimeMs=150)
    pt.Render(sc)
    n = int(sc.FrameBuffer.MetaData["NumIterations"])
    assert 1 <= n < 100000
    assert pt.last_stats.renderTimeMs <= 150 * 1.5 + 50
    limited = sc.FrameBuffer.Image.data.copy()
    sc.FrameBuffer.Reset()
    PathTracer(TotalSpp=n, MaxDepth=6, EnableDenoiser=False).Render(sc)
    assert np.array_equal(sc.FrameBuffer.Image.data, limited)
