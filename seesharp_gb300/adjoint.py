"""Differentiable rendering: the path-replay adjoint behind a forward/backward API.

`DifferentiableRender` binds a prepared Scene, a PathTracer and a set of parameters (one RGB
texture, the constant roughness of some GenericMaterials, and the radiance of some emitters).
`forward(texture, roughness, radiance)` uploads the parameters and renders (sst_forward);
`backward(dLoss/dImage)` replays every path from its RNG seed and returns dLoss/dparams
(sst_backward).  `RenderFunction` wraps the pair as a torch.autograd.Function.
"""
from __future__ import annotations

import numpy as np

from . import _native
from .images import RgbColor


class DifferentiableRender:
    def __init__(self, scene, integrator, texture=None, roughness_materials=(), emitters=(), views=None):
        """texture: the TextureRgb whose image is a parameter (or None); roughness_materials:
        GenericMaterials whose constant roughness is a parameter; emitters: list of groups, each a
        list of Emitter objects sharing one RGB radiance parameter; views: None (the scene's
        camera) or a list of (worldToCamera, fov) camera views rendered in one batch, in which
        case forward returns one image per view and backward takes one dLoss/dImage per view."""
        self.scene = scene
        self.pt = integrator
        self.texture = texture
        self.rough_mats = list(roughness_materials)
        self.emitter_groups = [list(g) for g in emitters]
        sc = scene.native
        self.tex_id = None if texture is None else sc._textures[(id(texture.Image), int(texture.Border))]
        self.mat_ids = [scene._mat_ids[id(m)] for m in self.rough_mats]
        self.em_ids = [[scene._emitter_index[id(e)] for e in g] for g in self.emitter_groups]
        self.params = integrator.params(scene)
        self.params.firstIteration = 0
        self.n_mat = len(scene._mat_ids)
        self.n_em = len(scene.Emitters)
        sizes = sc.texture_sizes
        self.n_tex = int(sum(sizes))
        self.tex_offset = None if self.tex_id is None else int(sum(sizes[:self.tex_id]))
        self.stats_forward = None
        self.stats_backward = None
        self.views = None if views is None else [_native.make_camera(m, f) for m, f in views]

    def set_parameters(self, texture=None, roughness=None, radiance=None):
        sc = self.scene.native
        if texture is not None and self.texture is not None:
            data = np.ascontiguousarray(texture, np.float32).reshape(self.texture.Image.data.shape)
            self.texture.Image.data[...] = data
            sc.update_texture(self.tex_id, data)
        if roughness is not None:
            for m, mid, r in zip(self.rough_mats, self.mat_ids, np.asarray(roughness, np.float32).reshape(-1)):
                m.MaterialParameters.Roughness.constColor = float(r)
                sc.update_generic(mid, m.MaterialParameters)
        if radiance is not None:
            rad = np.asarray(radiance, np.float32).reshape(-1, 3)
            for g, ids, r in zip(self.emitter_groups, self.em_ids, rad):
                for e, k in zip(g, ids):
                    e.Radiance = RgbColor(r)
                    sc.set_emitter_radiance(k, r)

    def _jobs(self, films):
        sh = self.scene.native
        return [(sh, self.params, f.ctypes.data, _native.SST_MEM_HOST, v) for f, v in zip(films, self.views)]

    def forward(self, texture=None, roughness=None, radiance=None):
        self.set_parameters(texture, roughness, radiance)
        fb = self.scene.FrameBuffer
        if self.views is not None:
            self._films = [np.zeros((fb.Height, fb.Width, 3), np.float32) for _ in self.views]
            self.stats_forward = _native.forward_batch(self.scene.native.ctx, self._jobs(self._films))
            return [f.copy() for f in self._films]
        film = np.zeros((fb.Height, fb.Width, 3), np.float32)
        self.stats_forward = self.scene.native.forward(self.params, film.ctypes.data)
        return film

    def backward(self, dloss_dimage):
        if self.views is not None:
            outs, st = _native.backward_batch(self.scene.native.ctx, self._jobs(self._films), dloss_dimage, self.n_tex, self.n_mat, self.n_em)
            g = outs[0]
        else:
            g, st = self.scene.native.backward(self.params, dloss_dimage, self.n_tex, self.n_mat, self.n_em)
        self.stats_backward = st
        out = {}
        if self.texture is not None:
            n = self.texture.Image.data.size
            out["texture"] = g["textures"][self.tex_offset:self.tex_offset + n].reshape(self.texture.Image.data.shape)
        out["roughness"] = g["materialRoughness"][self.mat_ids] if self.mat_ids else np.zeros(0, np.float32)
        out["radiance"] = np.array([g["emitterRadiance"][ids].sum(axis=0) for ids in self.em_ids], np.float32).reshape(-1, 3)
        out["raw"] = g
        return out


def render_function():
    """torch.autograd.Function over a DifferentiableRender (imported lazily: torch is plumbing)."""
    import torch

    class RenderFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, dr, texture, roughness, radiance):
            img = dr.forward(texture.detach().cpu().numpy(), roughness.detach().cpu().numpy(), radiance.detach().cpu().numpy())
            ctx.dr = dr
            return torch.from_numpy(img).to(texture.device)

        @staticmethod
        def backward(ctx, grad):
            g = ctx.dr.backward(grad.detach().cpu().numpy())
            dev = grad.device
            return None, torch.from_numpy(g["texture"]).to(dev), torch.from_numpy(g["roughness"]).to(dev), torch.from_numpy(g["radiance"]).to(dev)

    return RenderFunction


def l2_loss(image, target):
    """Mean squared error over pixels and channels (float64) and its gradient dLoss/dImage (float32)."""
    d = np.asarray(image, np.float64) - np.asarray(target, np.float64)
    return float(np.mean(d * d)), (2.0 * d / d.size).astype(np.float32)
