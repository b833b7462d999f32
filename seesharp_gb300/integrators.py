"""Integrator plugin API and the GPU PathTracer.

Mirrors SeeSharp's abstract Integrator (Integrators/Integrator.cs:6-30) and the public settings of
PathTracerBase (Integrators/PathTracer.cs:16-49).  Render() runs the whole progressive loop on the
GPU through sst_render; the per-event observer hooks of the reference are not called per path.
A subclass that overrides a behaviour-changing hook is rejected, because the GPU kernels cannot
run Python code per path (the reference's hooks at PathTracer.cs:277-530).
"""
from __future__ import annotations

import os

import numpy as np

from . import _native
from .images import MonochromeImage, OutlierReplayCache, RgbColor, RgbImage, RgbLayer


class Integrator:
    """Integrators/Integrator.cs:6-30."""

    def __init__(self):
        self.MaxDepth = 100
        self.MinDepth = 1

    def Render(self, scene):
        raise NotImplementedError


_BEHAVIOUR_HOOKS = ("ComputeSurvivalProbability", "RenderPixel", "EstimateIncidentRadiance", "OnBackgroundHit", "OnLightHit",
                    "PerformBackgroundNextEvent", "PerformNextEventEstimation", "DirectionPdf", "SampleDirection")


class PathTracer(Integrator):
    """Unidirectional path tracer with next-event estimation and balance-heuristic MIS."""

    def __init__(self, **kw):
        super().__init__()
        self.BaseSeed = 0xC030114
        self.TotalSpp = 20
        self.MaximumRenderTimeMs = None
        self.NumShadowRays = 1
        self.EnableBsdfDI = True
        self.RenderTechniquePyramid = False
        # The reference logs the denoiser's albedo / normal layers and denoises the last iteration
        # with Open Image Denoise by default; the layers are computed on the GPU, the denoiser is
        # outside this library.
        self.EnableDenoiser = True
        # ShadingStats (Shading/ShadingStats.cs): the reference counts every material call in every
        # render.  Here counting is a switch (it traces the shadow rays of next-event samples that
        # contribute nothing, whose visibility decides the reference's counts); with it on, Render
        # writes FrameBuffer.MetaData["ShadingStats"] as PathTracer.cs:256 does.
        self.CountShadingStats = False
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)

    # Behaviour-changing hooks exist so that overriding them can be detected.
    def ComputeSurvivalProbability(self, *a):
        raise NotImplementedError

    RenderPixel = EstimateIncidentRadiance = OnBackgroundHit = OnLightHit = ComputeSurvivalProbability
    PerformBackgroundNextEvent = PerformNextEventEstimation = DirectionPdf = SampleDirection = ComputeSurvivalProbability

    def _check_hooks(self):
        for name in _BEHAVIOUR_HOOKS:
            if getattr(type(self), name) is not getattr(PathTracer, name):
                raise NotImplementedError(f"PathTracer.{name} is overridden; the GPU path tracer runs the reference behaviour only")

    def params(self, scene):
        fb = scene.FrameBuffer
        return _native.make_params(fb.Width, fb.Height, int(self.TotalSpp), int(self.MaxDepth), int(self.MinDepth), int(self.BaseSeed),
                                   int(self.NumShadowRays), bool(self.EnableBsdfDI), fb.IgnoreNanAndInf, int(fb.CurIteration),
                                   int(self.MaximumRenderTimeMs or 0))

    def Render(self, scene):
        """PathTracerBase.Render (PathTracer.cs:199-267): TotalSpp iterations into scene.FrameBuffer."""
        self._check_hooks()
        fb = scene.FrameBuffer
        p = self.params(scene)
        if fb.CurIteration >= self.TotalSpp:
            return
        film = fb.Image.data
        assert film.dtype == np.float32 and film.flags["C_CONTIGUOUS"]
        if self.EnableDenoiser:
            # DenoiseBuffers (Integrators/Util/DenoiseBuffers.cs:10-15): the feature layers; the
            # denoiser itself (Open Image Denoise) is outside this library
            for name in ("albedo", "normal"):
                if name not in fb.layers:
                    fb.AddLayer(name, RgbLayer())
        albedo = fb.layers["albedo"].Image.data if "albedo" in fb.layers else None
        normal = fb.layers["normal"].Image.data if "normal" in fb.layers else None
        var = fb.PixelVariance
        pyramid = None
        if self.RenderTechniquePyramid:
            # PathTracer.cs:204-209: new pyramids for every Render call
            pyramid = np.zeros((2, 2 * int(self.MaxDepth), fb.Height, fb.Width, 3), np.float32)
        if fb.CurIteration == 0 or fb.OutlierCache is None:
            # FrameBuffer.Initialize (FrameBuffer.cs:229): a fresh cache with the first iteration
            fb.OutlierCache = OutlierReplayCache(fb.Width, fb.Height, fb.NumOutliersToTrack)
        oc = fb.OutlierCache
        outliers = (oc.weight, oc.iteration) if oc.nMax > 0 else None
        if self.CountShadingStats:
            _native.set_shading_stats(scene.native.ctx, True)
        try:
            stats = self._render(scene, p, film, var, albedo, normal, outliers, pyramid)
        finally:
            if self.CountShadingStats:
                _native.set_shading_stats(scene.native.ctx, False)
        self._finish(scene, stats, pyramid)

    def _render(self, scene, p, film, var, albedo, normal, outliers, pyramid):
        fb = scene.FrameBuffer
        if var is not None or fb.ReferenceImage is not None or albedo is not None or outliers is not None or pyramid is not None:
            ref = None if fb.ReferenceImage is None else fb.ReferenceImage.data
            stats, vimg, avg, err = scene.native.render_layers(p, film.ctypes.data, variance_state=None if var is None else var.state,
                                                               reference=ref, albedo=albedo, normal=normal, outliers=outliers, pyramid=pyramid)
            if var is not None:
                var.Image = MonochromeImage(vimg)
                var.Average = avg
            if err is not None:
                # per-iteration times are not separable in the wavefront: the render time is prorated
                n = int(stats.numIterations)
                fb.Errors += [(int(round(stats.renderTimeMs * (k + 1) / max(n, 1))), float(err[k, 0]), float(err[k, 1]), float(err[k, 2]))
                              for k in range(n)]
        else:
            stats = scene.native.render(p, film.ctypes.data)
        return stats

    def _finish(self, scene, stats, pyramid):
        fb = scene.FrameBuffer
        fb.CurIteration = fb.CurIteration + stats.numIterations
        fb.MetaData["NumIterations"] = fb.CurIteration
        fb.MetaData["RenderTime"] = stats.renderTimeMs
        fb.MetaData["FrameBufferTime"] = stats.frameBufferTimeMs
        fb.MetaData["RayTracerStats"] = {"NumRays": int(stats.numRays), "NumShadowRays": int(stats.numShadowRays)}
        if self.CountShadingStats:
            fb.MetaData["ShadingStats"] = {"NumMaterialEval": int(stats.numMaterialEval), "NumMaterialSample": int(stats.numMaterialSample),
                                           "NumMaterialPdf": int(stats.numMaterialPdf)}
        for k in range(min(4, int(stats.numNanOrInf))):
            px = stats.nanPixel[k]
            if px >= 0:
                fb.NaNWarnings.append((px % fb.Width, px // fb.Width, stats.nanIteration[k]))
        fb.MetaData["NumNaNOrInf"] = int(stats.numNanOrInf)
        self.last_stats = stats
        if pyramid is not None:
            # PathTracer.cs:261-266
            self.techPyramidRaw = TechPyramid(int(self.MinDepth), int(self.MaxDepth), pyramid[0])
            self.techPyramidWeighted = TechPyramid(int(self.MinDepth), int(self.MaxDepth), pyramid[1])
            self.techPyramidRaw.WriteToFiles(os.path.join(fb.Basename, "techs-raw"))
            self.techPyramidWeighted.WriteToFiles(os.path.join(fb.Basename, "techs-weighted"))

    def ReplayPixel(self, scene, pixel, iteration):
        """PathTracerBase.ReplayPixel (PathTracer.cs:60-68): re-renders the path of `pixel` (a Pixel or
        (col, row)) in the 0-based `iteration` from its seed and returns (graph, estimate).  The path
        graph is a debugging aid of the reference that is not built here (None)."""
        self._check_hooks()
        col, row = pixel
        fb = scene.FrameBuffer
        if not (0 <= col < fb.Width and 0 <= row < fb.Height):
            raise ValueError("pixel outside the frame buffer")
        p = self.params(scene)
        rgb, _ = scene.native.render_paths(p, [row * fb.Width + col], [int(iteration)])
        return None, RgbColor(*rgb[0])


class TechPyramid:
    """Integrators/Bidir/TechPyramid.cs as the PathTracer builds it (no merges, connections or light
    tracing): per path length d in [minDepth, maxDepth] the images of the techniques "{d}-hit" and,
    for d >= 2, "{d}-next-event".  `layers` is one pyramid as the GPU fills it, (2*maxDepth, H, W, 3)
    with layer 2(d-1) the hit technique and 2(d-1)+1 the next-event one."""

    def __init__(self, minDepth, maxDepth, layers):
        self.minDepth, self.maxDepth = int(minDepth), int(maxDepth)
        self.techniqueNames = {}
        self.techniqueImages = {}
        for depth in range(self.minDepth, self.maxDepth + 1):
            self.techniqueNames[(depth, 0, depth)] = f"{depth}-hit"
            self.techniqueImages[(depth, 0, depth)] = RgbImage(np.ascontiguousarray(layers[2 * (depth - 1)]))
            if depth == 1:
                continue
            self.techniqueNames[(depth - 1, 0, depth)] = f"{depth}-next-event"
            self.techniqueImages[(depth - 1, 0, depth)] = RgbImage(np.ascontiguousarray(layers[2 * (depth - 1) + 1]))

    def GetImagesForPathLength(self, totalEdges):
        return [(self.techniqueNames[k], img) for k, img in self.techniqueImages.items() if k[2] == totalEdges]

    def Normalize(self, scalingFactor):
        for img in self.techniqueImages.values():
            img.Scale(scalingFactor)

    def WriteToFiles(self, basename):
        """One layered OpenEXR file per path length, "<basename>-depth-<d>.exr", a layer per
        technique (channels "<technique>.R/G/B")."""
        from .imagefile import write_exr
        d = os.path.dirname(basename)
        if d:
            os.makedirs(d, exist_ok=True)
        for depth in range(self.minDepth, self.maxDepth + 1):
            ch = {}
            for name, img in self.GetImagesForPathLength(depth):
                for c, k in zip("RGB", range(3)):
                    ch[f"{name}.{c}"] = img.data[:, :, k]
            write_exr(f"{basename}-depth-{depth}.exr", ch)


def autotune(scene, integrator, trial_iterations=2):
    """Chooses the launch configuration (wave capacity, traversal block size, shared stack
    entries, resident traversal blocks) for rendering `scene` with `integrator` by timing short
    trial renders, and applies it to the scene's device context.  Images do not depend on it."""
    integrator._check_hooks()
    return _native.autotune(scene.native, integrator.params(scene), trial_iterations)


def render_batch(pairs):
    """Renders many (scene, PathTracer) pairs in one shared wavefront (sst_render_batch).

    Every scene must be prepared on the same device.  The films are the scenes' FrameBuffers,
    exactly as if each PathTracer had rendered its scene alone.
    """
    if not pairs:
        return None
    ctx = pairs[0][0].native.ctx
    jobs = []
    for sc, pt in pairs:
        pt._check_hooks()
        if sc.native.ctx is not ctx:
            raise ValueError("all scenes of a batch must share one device context")
        p = pt.params(sc)
        film = sc.FrameBuffer.Image.data
        jobs.append((sc.native, p, film.ctypes.data, _native.SST_MEM_HOST))
    stats = _native.render_batch(ctx, jobs)
    for sc, pt in pairs:
        fb = sc.FrameBuffer
        fb.CurIteration = max(fb.CurIteration, int(pt.TotalSpp))
        fb.MetaData["NumIterations"] = fb.CurIteration
    return stats
