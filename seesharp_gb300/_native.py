"""ctypes binding of libsst.so (declarations in include/sst.h).

The library is built in-tree by seesharp_gb300/build.py.  Loading fails loudly when it is
missing or when no CUDA device can be opened: there is no CPU fallback behind this package.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsst.so")

SST_MEM_HOST = 0
SST_MEM_DEVICE = 1
SST_NOALLOC_MAX_RAYS = 65536  # rays per sst_occluded_noalloc call

_ERRORS = {
    -1: "invalid argument",
    -2: "invalid scene",
    -3: "CUDA error",
    -4: "out of memory",
    -5: "scene not committed",
    -6: "device limit reached",
    -7: "unsupported",
}


class SstError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"libsst error {code} ({_ERRORS.get(code, '?')}): {message}")
        self.code = code


class SstGenericMaterial(ctypes.Structure):
    _fields_ = [("baseColor", ctypes.c_float * 3), ("baseColorTexture", ctypes.c_int32), ("roughness", ctypes.c_float),
                ("roughnessTexture", ctypes.c_int32), ("metallic", ctypes.c_float), ("specularTintStrength", ctypes.c_float),
                ("anisotropic", ctypes.c_float), ("specularTransmittance", ctypes.c_float), ("indexOfRefraction", ctypes.c_float)]


class SstRay(ctypes.Structure):
    _fields_ = [("org", ctypes.c_float * 3), ("tmin", ctypes.c_float), ("dir", ctypes.c_float * 3), ("tmax", ctypes.c_float)]


class SstHit(ctypes.Structure):
    _fields_ = [("distance", ctypes.c_float), ("u", ctypes.c_float), ("v", ctypes.c_float), ("primId", ctypes.c_int32),
                ("meshId", ctypes.c_int32), ("errorOffset", ctypes.c_float), ("position", ctypes.c_float * 3),
                ("normal", ctypes.c_float * 3)]


class SstPathTracerParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("totalSpp", ctypes.c_int32), ("maxDepth", ctypes.c_int32),
                ("minDepth", ctypes.c_int32), ("baseSeed", ctypes.c_uint32), ("numShadowRays", ctypes.c_int32),
                ("enableBsdfDI", ctypes.c_int32), ("ignoreNanAndInf", ctypes.c_int32), ("firstIteration", ctypes.c_int32),
                ("maximumRenderTimeMs", ctypes.c_int64)]


class SstRenderStats(ctypes.Structure):
    _fields_ = [("renderTimeMs", ctypes.c_double), ("frameBufferTimeMs", ctypes.c_double), ("numIterations", ctypes.c_int32),
                ("numKernelLaunches", ctypes.c_int32), ("numRays", ctypes.c_uint64), ("numShadowRays", ctypes.c_uint64),
                ("numNanOrInf", ctypes.c_uint64), ("nanPixel", ctypes.c_int32 * 4), ("nanIteration", ctypes.c_int32 * 4),
                ("numMaterialEval", ctypes.c_uint64), ("numMaterialSample", ctypes.c_uint64), ("numMaterialPdf", ctypes.c_uint64)]


class SstGradients(ctypes.Structure):
    _fields_ = [("textures", ctypes.c_void_p), ("materialBaseColor", ctypes.c_void_p), ("materialRoughness", ctypes.c_void_p),
                ("emitterRadiance", ctypes.c_void_p), ("memory", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class SstTuning(ctypes.Structure):
    _fields_ = [("waveCapacity", ctypes.c_int32), ("traceBlock", ctypes.c_int32), ("traceStackShared", ctypes.c_int32),
                ("traceBlocksPerSM", ctypes.c_int32), ("traceBvhWidth", ctypes.c_int32), ("traceRefillIdle", ctypes.c_int32),
                ("shadeBlocks", ctypes.c_int32), ("shadeOrder", ctypes.c_int32), ("shadeSplit", ctypes.c_int32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class SstFilmLayers(ctypes.Structure):
    _fields_ = [("variance", ctypes.c_void_p), ("varianceAverage", ctypes.c_void_p), ("varianceState", ctypes.c_void_p), ("reference", ctypes.c_void_p),
                ("errors", ctypes.c_void_p), ("albedo", ctypes.c_void_p), ("normal", ctypes.c_void_p), ("memory", ctypes.c_int32),
                ("numOutliers", ctypes.c_int32), ("outlierWeight", ctypes.c_void_p), ("outlierIteration", ctypes.c_void_p),
                ("techPyramid", ctypes.c_void_p)]


class SstCamera(ctypes.Structure):
    _fields_ = [("worldToCamera", ctypes.c_float * 16), ("verticalFovDegrees", ctypes.c_float), ("reserved", ctypes.c_int32)]


class SstRenderJob(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("params", SstPathTracerParams), ("film", ctypes.c_void_p), ("memory", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("camera", ctypes.POINTER(SstCamera))]


# Every exported symbol with its argument types (restype int unless noted).
_P = ctypes.POINTER
_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_u32 = ctypes.c_uint32
_f = ctypes.c_float
_fp = _P(ctypes.c_float)
SIGNATURES = {
    "sst_version": [_P(_i32), _P(_i32)],
    "sst_last_error": [ctypes.c_char_p, ctypes.c_size_t],
    "sst_create": [_i32, _P(_vp)],
    "sst_destroy": [_vp],
    "sst_scene_create": [_vp, _P(_vp)],
    "sst_scene_destroy": [_vp],
    "sst_scene_add_texture": [_vp, _vp, _i32, _i32, _i32, _i32, _P(_i32)],
    "sst_scene_add_material_diffuse": [_vp, _fp, _i32, _i32, _P(_i32)],
    "sst_scene_add_material_generic": [_vp, _P(SstGenericMaterial), _P(_i32)],
    "sst_scene_update_material_generic": [_vp, _i32, _P(SstGenericMaterial)],
    "sst_scene_add_mesh": [_vp, _vp, _i32, _vp, _i32, _vp, _vp, _i32, _P(_i32)],
    "sst_scene_add_emitters": [_vp, _i32, _vp, _i32, _fp, _f, _P(_i32), _P(_i32)],
    "sst_scene_set_emitter_radiance": [_vp, _i32, _i32, _vp],
    "sst_scene_set_envmap": [_vp, _vp, _i32, _i32],
    "sst_scene_set_camera": [_vp, _fp, _f],
    "sst_scene_commit": [_vp, _i32, _i32],
    "sst_scene_info": [_vp, _P(_i32), _P(_i32), _P(_i32)],
    "sst_trace": [_vp, _vp, _i32, _vp, _i32],
    "sst_occluded": [_vp, _vp, _i32, _vp, _i32],
    "sst_occluded_noalloc": [_vp, _vp, _i32, _vp, _i32],
    "sst_render": [_vp, _P(SstPathTracerParams), _vp, _i32, _P(SstRenderStats)],
    "sst_render_batch": [_vp, _P(SstRenderJob), _i32, _P(SstRenderStats)],
    "sst_scene_update_texture": [_vp, _i32, _vp],
    "sst_forward_batch": [_vp, _vp, _i32, _P(SstRenderStats)],
    "sst_trace_light_paths": [_vp, ctypes.c_uint32, ctypes.c_uint32, _i32, _i32, _vp, _vp, _i32, _P(SstRenderStats)],
    "sst_render_layers": [_vp, _P(SstPathTracerParams), _vp, _i32, _P(SstFilmLayers), _P(SstRenderStats)],
    "sst_render_paths": [_vp, _P(SstPathTracerParams), _vp, _vp, _i32, _vp, _i32, _P(SstRenderStats)],
    "sst_backward_batch": [_vp, _vp, _i32, _vp, _i32, _vp, _P(SstRenderStats)],
    "sst_forward": [_vp, _P(SstPathTracerParams), _vp, _i32, _P(SstRenderStats)],
    "sst_backward": [_vp, _P(SstPathTracerParams), _vp, _i32, _P(SstGradients), _P(SstRenderStats)],
    "sst_get_tuning": [_vp, _P(SstTuning)],
    "sst_set_tuning": [_vp, _P(SstTuning)],
    "sst_autotune": [_vp, _P(SstPathTracerParams), _i32, _P(SstTuning), _P(ctypes.c_double)],
    "sst_set_profiling": [_vp, _i32],
    "sst_set_shading_stats": [_vp, _i32],
    "sst_get_kernel_times": [_vp, _vp, _vp, _vp, _i32],
    "sst_debug_material_eval": [_vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp],
    "sst_debug_material_sample": [_vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp],
    "sst_debug_envmap": [_vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "sst_debug_rng": [_u32, _u32, _i32, _vp, _i32, _vp],
    "sst_debug_camera": [_vp, _i32, _vp, _vp, _vp],
}

_lib = None
_lib_lock = threading.Lock()


def load_library(path=None):
    """Loads libsst.so and declares its prototypes.  Raises if the library is absent."""
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise ImportError(f"libsst.so not found at {p}; build it with `python -m seesharp_gb300.build`")
        lib = ctypes.CDLL(p)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = lib
        return lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    load_library().sst_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(code):
    if code != 0:
        raise SstError(code, last_error())
    return code


def ptr(a):
    """Host pointer of a contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


def fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class Context:
    """An sst_ctx on one CUDA device."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        check(self.lib.sst_create(int(device), ctypes.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self.lib.sst_destroy(self.handle)
            self.handle = None


_contexts = {}


def default_context(device=0):
    ctx = _contexts.get(device)
    if ctx is None:
        ctx = Context(device)
        _contexts[device] = ctx
    return ctx


KERNEL_CLASSES = ["camera", "trace_closest", "shade", "trace_shadow", "film_fold"]


def set_profiling(ctx, enable):
    check(ctx.lib.sst_set_profiling(ctx.handle, int(bool(enable))))


def set_shading_stats(ctx, enable):
    """Counts the reference's material calls (ShadingStats) in the context's renders (sst_set_shading_stats)."""
    check(ctx.lib.sst_set_shading_stats(ctx.handle, int(bool(enable))))


def get_tuning(ctx):
    t = SstTuning()
    check(ctx.lib.sst_get_tuning(ctx.handle, ctypes.byref(t)))
    return t.as_dict()


def set_tuning(ctx, **kw):
    """Changes the named fields of the context's launch configuration (SstTuning)."""
    t = SstTuning()
    check(ctx.lib.sst_get_tuning(ctx.handle, ctypes.byref(t)))
    for k, v in kw.items():
        if k not in dict(SstTuning._fields_):
            raise AttributeError(k)
        setattr(t, k, int(v))
    check(ctx.lib.sst_set_tuning(ctx.handle, ctypes.byref(t)))


def autotune(scene_handle, params, trial_iterations=2):
    """sst_autotune: returns (chosen tuning as a dict, best trial time in ms)."""
    t = SstTuning()
    ms = ctypes.c_double()
    check(scene_handle.lib.sst_autotune(scene_handle.handle, ctypes.byref(params), int(trial_iterations), ctypes.byref(t), ctypes.byref(ms)))
    return t.as_dict(), ms.value


def kernel_times(ctx):
    n = len(KERNEL_CLASSES)
    ms = np.zeros(n, np.float64)
    la = np.zeros(n, np.int64)
    it = np.zeros(n, np.int64)
    check(ctx.lib.sst_get_kernel_times(ctx.handle, ptr(ms), ptr(la), ptr(it), n))
    return {k: {"ms": float(ms[i]), "launches": int(la[i]), "items": int(it[i])} for i, k in enumerate(KERNEL_CLASSES)}


class SceneHandle:
    """An sst_scene: thin wrappers of the sst_scene_* calls for the Python scene model."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.lib = ctx.lib
        h = ctypes.c_void_p()
        check(self.lib.sst_scene_create(ctx.handle, ctypes.byref(h)))
        self.handle = h
        self._textures = {}
        self.texture_sizes = []   # floats per texture, in id order (the gradient pool's layout)

    def close(self):
        if self.handle:
            self.lib.sst_scene_destroy(self.handle)
            self.handle = None

    # -- textures and materials --
    def add_texture(self, image, border):
        key = (id(image), int(border))
        if key in self._textures:
            return self._textures[key]
        d = np.ascontiguousarray(image.data, np.float32)
        out = ctypes.c_int32()
        check(self.lib.sst_scene_add_texture(self.handle, ptr(d), d.shape[1], d.shape[0], d.shape[2], int(border), ctypes.byref(out)))
        self._textures[key] = out.value
        self.texture_sizes.append(d.size)
        return out.value

    def _tex_rgb(self, tex):
        if tex.Image is None:
            return tex.constColor.array(), -1
        return np.zeros(3, np.float32), self.add_texture(tex.Image, tex.Border)

    def _tex_mono(self, tex):
        if tex.Image is None:
            return tex.constColor, -1
        return 0.0, self.add_texture(tex.Image, tex.Border)

    def generic_params(self, p):
        s = SstGenericMaterial()
        c, t = self._tex_rgb(p.BaseColor)
        s.baseColor[:] = [float(x) for x in c]
        s.baseColorTexture = t
        r, rt = self._tex_mono(p.Roughness)
        s.roughness = r
        s.roughnessTexture = rt
        s.metallic = p.Metallic
        s.specularTintStrength = p.SpecularTintStrength
        s.anisotropic = p.Anisotropic
        s.specularTransmittance = p.SpecularTransmittance
        s.indexOfRefraction = p.IndexOfRefraction
        return s

    def add_material(self, mat):
        from .scene import DiffuseMaterial, GenericMaterial
        out = ctypes.c_int32()
        if isinstance(mat, DiffuseMaterial):
            c, t = self._tex_rgb(mat.MaterialParameters.BaseColor)
            c = np.ascontiguousarray(c, np.float32)
            check(self.lib.sst_scene_add_material_diffuse(self.handle, fptr(c), t, int(mat.MaterialParameters.Transmitter), ctypes.byref(out)))
        elif isinstance(mat, GenericMaterial):
            s = self.generic_params(mat.MaterialParameters)
            check(self.lib.sst_scene_add_material_generic(self.handle, ctypes.byref(s), ctypes.byref(out)))
        else:
            raise TypeError(f"unsupported material type {type(mat).__name__}")
        return out.value

    def update_generic(self, material_id, params):
        s = self.generic_params(params)
        check(self.lib.sst_scene_update_material_generic(self.handle, int(material_id), ctypes.byref(s)))

    def add_mesh(self, mesh, material_id):
        out = ctypes.c_int32()
        check(self.lib.sst_scene_add_mesh(self.handle, ptr(mesh.Vertices), mesh.NumVertices, ptr(mesh.Indices), mesh.NumFaces,
                                          ptr(mesh.ShadingNormals), ptr(mesh.TextureCoordinates), int(material_id), ctypes.byref(out)))
        return out.value

    def add_emitters(self, mesh_id, faces, radiance, exponent):
        first, count = ctypes.c_int32(), ctypes.c_int32()
        rad = np.ascontiguousarray(radiance, np.float32)
        fa = None if faces is None else np.ascontiguousarray(faces, np.int32)
        n = 0 if fa is None else fa.size
        check(self.lib.sst_scene_add_emitters(self.handle, int(mesh_id), ptr(fa), n, fptr(rad), float(exponent), ctypes.byref(first),
                                              ctypes.byref(count)))
        return first.value

    def set_emitter_radiance(self, first, rgb):
        rgb = np.ascontiguousarray(rgb, np.float32).reshape(-1, 3)
        check(self.lib.sst_scene_set_emitter_radiance(self.handle, int(first), rgb.shape[0], ptr(rgb)))

    def set_envmap(self, data):
        d = np.ascontiguousarray(data, np.float32)
        check(self.lib.sst_scene_set_envmap(self.handle, ptr(d), d.shape[1], d.shape[0]))

    def set_camera(self, m, fov):
        mm = np.ascontiguousarray(np.asarray(m, np.float32).reshape(16))
        check(self.lib.sst_scene_set_camera(self.handle, fptr(mm), float(fov)))

    def commit(self, width, height):
        check(self.lib.sst_scene_commit(self.handle, int(width), int(height)))

    def info(self):
        a, b, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        check(self.lib.sst_scene_info(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"emitters": a.value, "triangles": b.value, "bvh_nodes": c.value}

    # -- queries --
    def trace(self, rays):
        """rays: (n, 8) float32 (org, tmin, dir, tmax) -> structured hits (n, 12) float32 view."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.zeros((rays.shape[0], 12), np.float32)
        check(self.lib.sst_trace(self.handle, ptr(rays), rays.shape[0], ptr(hits), SST_MEM_HOST))
        return hits

    def occluded(self, rays):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        occ = np.zeros(rays.shape[0], np.int32)
        check(self.lib.sst_occluded(self.handle, ptr(rays), rays.shape[0], ptr(occ), SST_MEM_HOST))
        return occ

    def occluded_noalloc(self, rays):
        """sst_occluded_noalloc: the same results as occluded(), without any device allocation;
        at most SST_NOALLOC_MAX_RAYS rays per call."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        occ = np.zeros(rays.shape[0], np.int32)
        check(self.lib.sst_occluded_noalloc(self.handle, ptr(rays), rays.shape[0], ptr(occ), SST_MEM_HOST))
        return occ

    def render_layers(self, params, film, variance_state=None, reference=None, albedo=None, normal=None, outliers=None, pyramid=None):
        """sst_render_layers into a host film.  variance_state: (2, H, W) float32 running means (in/out)
        or None; albedo / normal: (H, W, 3) float32 layers (in/out) or None; outliers: a pair of
        (H, W, n) float32 heap priorities and int32 heap iterations (in/out) or None; pyramid: a
        float32 (2, 2*maxDepth, H, W, 3) array for the technique pyramids (out) or None.  Returns (stats,
        variance image or None, variance average or None, (iterations of this call, 3) array of
        (MSE, RelMSE, RelMSE_Outlier) or None)."""
        W, H = params.width, params.height
        L = SstFilmLayers()
        var = np.zeros((H, W), np.float32) if variance_state is not None else None
        avg = np.zeros(1, np.float32) if variance_state is not None else None
        ref = None if reference is None else np.ascontiguousarray(reference, np.float32)
        err = np.zeros((max(0, params.totalSpp - params.firstIteration), 3), np.float64) if reference is not None else None
        ow, oi = outliers if outliers is not None else (None, None)
        for name, arr in (("variance", var), ("varianceAverage", avg), ("varianceState", variance_state), ("reference", ref), ("errors", err),
                          ("albedo", albedo), ("normal", normal), ("outlierWeight", ow), ("outlierIteration", oi), ("techPyramid", pyramid)):
            if arr is not None:
                assert arr.flags["C_CONTIGUOUS"]
                setattr(L, name, arr.ctypes.data)
        if pyramid is not None:
            assert pyramid.dtype == np.float32 and pyramid.shape == (2, 2 * params.maxDepth, H, W, 3)
        if outliers is not None:
            assert ow.dtype == np.float32 and oi.dtype == np.int32 and ow.shape == oi.shape == (H, W, ow.shape[2])
            L.numOutliers = ow.shape[2]
        L.memory = SST_MEM_HOST
        stats = SstRenderStats()
        check(self.lib.sst_render_layers(self.handle, ctypes.byref(params), ctypes.c_void_p(film), SST_MEM_HOST, ctypes.byref(L), ctypes.byref(stats)))
        return stats, var, None if avg is None else float(avg[0]), err

    def render_paths(self, params, pixels, iterations):
        """sst_render_paths: the estimates (n, 3) float32 of the paths (pixels[k], iterations[k])."""
        px = np.ascontiguousarray(pixels, np.int32).reshape(-1)
        it = np.ascontiguousarray(iterations, np.int32).reshape(-1)
        if px.shape != it.shape:
            raise ValueError("pixels and iterations differ in length")
        rgb = np.zeros((px.size, 3), np.float32)
        stats = SstRenderStats()
        check(self.lib.sst_render_paths(self.handle, ctypes.byref(params), ptr(px), ptr(it), px.size, ptr(rgb), SST_MEM_HOST, ctypes.byref(stats)))
        return rgb, stats

    def trace_light_paths(self, seed, iteration, num_paths, max_depth):
        """sst_trace_light_paths: (floats (n, maxDepth+1, 16), ints (n, maxDepth+1, 6), lengths (n,),
        stats) in the layout of SstPathVertex."""
        stride = max_depth + 1
        raw = np.zeros((num_paths, stride, 22), np.float32)
        lengths = np.zeros(num_paths, np.int32)
        stats = SstRenderStats()
        check(self.lib.sst_trace_light_paths(self.handle, seed & 0xFFFFFFFF, iteration & 0xFFFFFFFF, int(num_paths), int(max_depth), ptr(raw),
                                              ptr(lengths), SST_MEM_HOST, ctypes.byref(stats)))
        return raw[..., :16].copy(), raw[..., 16:].copy().view(np.int32), lengths, stats

    def update_texture(self, tex_id, data):
        d = np.ascontiguousarray(data, np.float32)
        check(self.lib.sst_scene_update_texture(self.handle, int(tex_id), ptr(d)))

    def forward(self, params, film, memory=SST_MEM_HOST):
        stats = SstRenderStats()
        check(self.lib.sst_forward(self.handle, ctypes.byref(params), ctypes.c_void_p(film), int(memory), ctypes.byref(stats)))
        return stats

    def backward(self, params, dldi, n_tex, n_mat, n_em, memory=SST_MEM_HOST):
        """dldi: (H, W, 3) float32 host array.  Returns host gradient arrays and the stats."""
        d = np.ascontiguousarray(dldi, np.float32)
        g = SstGradients()
        out = {"textures": np.zeros(max(n_tex, 1), np.float32), "materialBaseColor": np.zeros(max(3 * n_mat, 1), np.float32),
               "materialRoughness": np.zeros(max(n_mat, 1), np.float32), "emitterRadiance": np.zeros(max(3 * n_em, 1), np.float32)}
        g.textures, g.materialBaseColor = out["textures"].ctypes.data, out["materialBaseColor"].ctypes.data
        g.materialRoughness, g.emitterRadiance = out["materialRoughness"].ctypes.data, out["emitterRadiance"].ctypes.data
        g.memory = SST_MEM_HOST
        stats = SstRenderStats()
        check(self.lib.sst_backward(self.handle, ctypes.byref(params), ptr(d), int(memory), ctypes.byref(g), ctypes.byref(stats)))
        out["textures"] = out["textures"][:n_tex]
        out["materialBaseColor"] = out["materialBaseColor"][:3 * n_mat].reshape(-1, 3)
        out["materialRoughness"] = out["materialRoughness"][:n_mat]
        out["emitterRadiance"] = out["emitterRadiance"][:3 * n_em].reshape(-1, 3)
        return out, stats

    def render(self, params, film, memory=SST_MEM_HOST):
        stats = SstRenderStats()
        check(self.lib.sst_render(self.handle, ctypes.byref(params), ctypes.c_void_p(film), int(memory), ctypes.byref(stats)))
        return stats


def make_camera(world_to_camera, fov):
    c = SstCamera()
    c.worldToCamera[:] = [float(x) for x in np.asarray(world_to_camera, np.float32).reshape(16)]
    c.verticalFovDegrees = float(fov)
    return c


def _job_array(jobs):
    """jobs: list of (SceneHandle, SstPathTracerParams, film_ptr, memory[, SstCamera or None])."""
    arr = (SstRenderJob * len(jobs))()
    keep = []
    for k, job in enumerate(jobs):
        sh, params, film, mem = job[:4]
        cam = job[4] if len(job) > 4 else None
        arr[k].scene = sh.handle
        arr[k].params = params
        arr[k].film = film
        arr[k].memory = mem
        if cam is not None:
            keep.append(cam)
            arr[k].camera = ctypes.pointer(cam)
    return arr, keep


def render_batch(ctx, jobs):
    """One shared wavefront over jobs (SceneHandle, params, film_ptr, memory[, camera view])."""
    arr, _keep = _job_array(jobs)
    stats = SstRenderStats()
    check(ctx.lib.sst_render_batch(ctx.handle, arr, len(jobs), ctypes.byref(stats)))
    return stats


def forward_batch(ctx, jobs):
    arr, _keep = _job_array(jobs)
    stats = SstRenderStats()
    check(ctx.lib.sst_forward_batch(ctx.handle, arr, len(jobs), ctypes.byref(stats)))
    return stats


def backward_batch(ctx, jobs, dldis, n_tex, n_mat, n_em):
    """dldis: one (H, W, 3) float32 host array per job.  Returns per distinct scene (in order of
    first appearance) the host gradient arrays, summed over the scene's jobs, and the stats."""
    arr, _keep = _job_array(jobs)
    ds = [np.ascontiguousarray(d, np.float32) for d in dldis]
    dp = (ctypes.c_void_p * len(ds))(*[d.ctypes.data for d in ds])
    grads = (SstGradients * len(jobs))()
    outs, seen = [], {}
    for k, job in enumerate(jobs):
        key = id(job[0])
        if key in seen:
            continue
        o = {"textures": np.zeros(max(n_tex, 1), np.float32), "materialBaseColor": np.zeros(max(3 * n_mat, 1), np.float32),
             "materialRoughness": np.zeros(max(n_mat, 1), np.float32), "emitterRadiance": np.zeros(max(3 * n_em, 1), np.float32)}
        g = grads[k]
        g.textures, g.materialBaseColor = o["textures"].ctypes.data, o["materialBaseColor"].ctypes.data
        g.materialRoughness, g.emitterRadiance = o["materialRoughness"].ctypes.data, o["emitterRadiance"].ctypes.data
        g.memory = SST_MEM_HOST
        seen[key] = len(outs)
        outs.append(o)
    stats = SstRenderStats()
    check(ctx.lib.sst_backward_batch(ctx.handle, arr, len(jobs), dp, SST_MEM_HOST, grads, ctypes.byref(stats)))
    for o in outs:
        o["textures"] = o["textures"][:n_tex]
        o["materialBaseColor"] = o["materialBaseColor"][:3 * n_mat].reshape(-1, 3)
        o["materialRoughness"] = o["materialRoughness"][:n_mat]
        o["emitterRadiance"] = o["emitterRadiance"][:3 * n_em].reshape(-1, 3)
    return outs, stats


def make_params(width, height, totalSpp, maxDepth, minDepth=1, baseSeed=0xC030114, numShadowRays=1, enableBsdfDI=True,
                ignoreNanAndInf=True, firstIteration=0, maximumRenderTimeMs=0):
    p = SstPathTracerParams()
    p.width, p.height, p.totalSpp, p.maxDepth, p.minDepth = width, height, totalSpp, maxDepth, minDepth
    p.baseSeed = baseSeed & 0xFFFFFFFF
    p.numShadowRays = numShadowRays
    p.enableBsdfDI = int(bool(enableBsdfDI))
    p.ignoreNanAndInf = int(bool(ignoreNanAndInf))
    p.firstIteration = firstIteration
    p.maximumRenderTimeMs = int(maximumRenderTimeMs or 0)
    return p
