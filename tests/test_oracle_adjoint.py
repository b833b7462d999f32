"""The oracle's FP64 path-replay adjoint against central differences of its own FP64 renders
(common random numbers).  For texels and emitter radiance the sampled paths and their pdfs do not
depend on the parameter (the textured back wall has no tinted or metallic specular part, so its
lobe-selection probabilities do not depend on the base colour), so the two agree to the rounding
of the FP32 film."""
import numpy as np

from oracle import pyoracle as O
from seesharp_gb300 import workloads
from seesharp_gb300.adjoint import l2_loss
from seesharp_gb300.images import RgbColor

W = H = 24
SPP = 2


def _scene():
    return workloads.cornell_box_differentiable(W, H, tex_res=8)


def _render(sc):
    o = O.OracleScene.from_scene(sc, fp64=True)
    return o.render(o.params(W, H, SPP, 5))[0]


def test_oracle_adjoint_matches_central_differences():
    sc, tex, boxes, lights = _scene()
    img = _render(sc)
    target = img * (1 + 0.2 * np.random.default_rng(0).standard_normal(img.shape))
    _, dldi = l2_loss(img, target)
    o = O.OracleScene.from_scene(sc, fp64=True)
    g = o.adjoint(o.params(W, H, SPP, 5), dldi, tex.Image.data.size, len(sc.Meshes), len(sc.Emitters))
    h = 1e-3
    tex0 = tex.Image.data.copy()
    fds, ads = [], []
    for e in (0, 5, 77, 100, 150, 191):
        vals = []
        for sgn in (1, -1):
            tex.Image.data[...] = tex0
            tex.Image.data.reshape(-1)[e] += sgn * h
            vals.append(l2_loss(_render(sc), target)[0])
        tex.Image.data[...] = tex0
        fds.append((vals[0] - vals[1]) / (2 * h))
        ads.append(g["textures"][e])
    # the FP32 film rounds each difference: compare the entries together (relative L2)
    fds, ads = np.array(fds), np.array(ads)
    assert np.linalg.norm(fds - ads) <= 5e-3 * np.linalg.norm(fds), (fds, ads)
    for c in range(3):
        vals = []
        for sgn in (1, -1):
            r = np.array([17.0, 12.0, 4.0])
            r[c] += sgn * h
            for em in lights:
                em.Radiance = RgbColor(*r)
            vals.append(l2_loss(_render(sc), target)[0])
        for em in lights:
            em.Radiance = RgbColor(17, 12, 4)
        fd = (vals[0] - vals[1]) / (2 * h)
        ad = g["emitterRadiance"][:, c].sum()
        assert abs(fd - ad) <= 2e-3 * abs(fd), (c, fd, ad)
