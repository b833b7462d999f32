"""The reference's own scene files, loaded by seesharp_gb300.sceneio, rendered by the CUDA path
and by the oracle on the same seeds: image means within 1% (SeeSharp.Validation/Validator.cs:26)
and per-path agreement."""
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from seesharp_gb300 import FrameBuffer, PathTracer, mean_rgb, sceneio

pytestmark = pytest.mark.gpu

SCENES = os.path.join(os.path.dirname(__file__), "golden", "scenes")


@pytest.mark.parametrize("name,spp,depth", [("CornellBox/CornellBox.json", 8, 5), ("simpledi.json", 8, 2), ("simplebackground.json", 8, 3),
                                            ("TextureTest/TextureTest.json", 8, 3), ("ExampleScene/ExampleScene.json", 8, 5)])
def test_reference_scene_renders_match_the_oracle(name, spp, depth):
    sc = sceneio.load_json_scene(os.path.join(SCENES, name))
    sc.FrameBuffer = FrameBuffer(96, 64)
    sc.Prepare()
    pt = PathTracer(TotalSpp=spp, MaxDepth=depth, BaseSeed=571298512)
    pt.Render(sc)
    g = sc.FrameBuffer.Image.data.copy()
    o = O.OracleScene.from_scene(sc)
    r, rays, _ = o.render(o.params(96, 64, spp, depth, baseSeed=571298512))
    assert np.isfinite(g).all() and mean_rgb(r) > 0
    assert abs(mean_rgb(g) - mean_rgb(r)) <= 0.01 * mean_rgb(r), (mean_rgb(g), mean_rgb(r))
    ok = np.all(np.abs(g - r) <= 1e-3 + 1e-2 * np.abs(r), axis=2).mean()
    assert ok >= 0.97, ok
    assert abs(int(pt.last_stats.numRays) - rays) <= 0.01 * rays
