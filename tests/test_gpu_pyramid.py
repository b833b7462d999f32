"""PathTracer.RenderTechniquePyramid (Integrators/PathTracer.cs:73-82, 204-266;
Integrators/Bidir/TechPyramid.cs): the per-technique images, raw and MIS-weighted, filled on the
GPU, against the oracle's restatement of RegisterSample."""
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from seesharp_gb300 import FrameBuffer, PathTracer, imagefile, workloads

pytestmark = pytest.mark.gpu


def _gpu(sc, **kw):
    sc.FrameBuffer.Reset()
    pt = PathTracer(RenderTechniquePyramid=True, EnableDenoiser=False, **kw)
    pt.Render(sc)
    return pt, sc.FrameBuffer.Image.data.copy()


def _layers(tp, max_depth, h, w):
    """(2*maxDepth, H, W, 3) from a TechPyramid, zero for techniques it does not have."""
    out = np.zeros((2 * max_depth, h, w, 3), np.float32)
    for (cam, _, depth), img in tp.techniqueImages.items():
        out[2 * (depth - 1) + (1 if cam == depth - 1 else 0)] = img.data
    return out


def _oracle(sc, spp, depth, **kw):
    o = O.OracleScene.from_scene(sc)
    p = o.params(sc.FrameBuffer.Width, sc.FrameBuffer.Height, spp, depth, **kw)
    return o.render_pyramid(p)


def _agree(a, b, rtol=1e-3, atol=2e-5):
    ok = np.all(np.abs(a - b) <= atol + rtol * np.abs(b), axis=-1)
    return ok.mean()


@pytest.mark.parametrize("max_depth", [4, 8])
def test_pyramid_matches_the_oracle(max_depth):
    """Every technique image, raw and weighted.  MaxDepth 8 brings in Russian roulette, which the
    reference leaves out of the next-event samples it registers (PathTracer.cs:443, 492)."""
    w, h, S = 40, 30, 4
    sc = workloads.cornell_box(w, h)
    sc.Prepare()
    pt, film = _gpu(sc, TotalSpp=S, MaxDepth=max_depth)
    got = np.stack([_layers(pt.techPyramidRaw, max_depth, h, w), _layers(pt.techPyramidWeighted, max_depth, h, w)])
    want = _oracle(sc, S, max_depth)
    for k in range(2):
        for L in range(2 * max_depth):
            assert _agree(got[k, L], want[k, L]) >= 0.98, (k, L, _agree(got[k, L], want[k, L]))
    assert np.abs(got[:, 1]).max() == 0  # there is no "1-next-event" technique
    if max_depth == 4:
        # without Russian roulette the weighted techniques sum to the image
        assert np.allclose(got[1].sum(axis=0), film, rtol=1e-4, atol=1e-5)


def test_pyramid_min_depth_shadow_rays_and_no_bsdf_di():
    """MinDepth 3: no technique below length 3.  Two shadow rays per vertex (the NS = 2 kernel).
    EnableBsdfDI off: hits beyond the first bounce carry MIS weight 0 but are still logged raw."""
    w, h, S, D = 32, 24, 3, 5
    sc = workloads.cornell_box(w, h)
    sc.Prepare()
    pt, _ = _gpu(sc, TotalSpp=S, MaxDepth=D, MinDepth=3, NumShadowRays=2, EnableBsdfDI=False)
    raw, wgt = _layers(pt.techPyramidRaw, D, h, w), _layers(pt.techPyramidWeighted, D, h, w)
    assert sorted(pt.techPyramidRaw.techniqueNames.values()) == ["3-hit", "3-next-event", "4-hit", "4-next-event", "5-hit", "5-next-event"]
    want = _oracle(sc, S, D, minDepth=3, numShadowRays=2, enableBsdfDI=False)
    assert np.abs(want[:, :4]).max() == 0
    for L in range(4, 2 * D):
        assert _agree(raw[L], want[0, L]) >= 0.98 and _agree(wgt[L], want[1, L]) >= 0.98, L
    for d in range(3, D + 1):
        assert np.abs(wgt[2 * (d - 1)]).max() == 0 and np.abs(raw[2 * (d - 1)]).max() > 0


def test_pyramid_files(tmp_path):
    """TechPyramid.WriteToFiles: "<Basename>/techs-raw-depth-<d>.exr" and the weighted ones, a layer
    per technique."""
    sc = workloads.cornell_box(16, 12)
    sc.FrameBuffer = FrameBuffer(16, 12, filename=str(tmp_path / "img.exr"))
    sc.Prepare()
    pt = PathTracer(TotalSpp=2, MaxDepth=3, RenderTechniquePyramid=True)
    pt.Render(sc)
    names = sorted(os.listdir(tmp_path / "img"))
    assert names == [f"techs-{k}-depth-{d}.exr" for k in ("raw", "weighted") for d in (1, 2, 3)]
    ch = imagefile.read_exr_channels(str(tmp_path / "img" / "techs-weighted-depth-2.exr"))
    assert sorted(ch) == ["2-hit.B", "2-hit.G", "2-hit.R", "2-next-event.B", "2-next-event.G", "2-next-event.R"]
    img = pt.techPyramidWeighted.techniqueImages[(1, 0, 2)].data
    assert np.array_equal(ch["2-next-event.G"], img[:, :, 1])
    assert sorted(imagefile.read_exr_channels(str(tmp_path / "img" / "techs-raw-depth-1.exr"))) == ["1-hit.B", "1-hit.G", "1-hit.R"]
