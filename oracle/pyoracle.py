"""ORACLE ctypes bridge -- test infrastructure only.

Loads oracle/liboracle.so (the CPU restatement of SeeSharp's PathTracer path) and realizes a
seesharp_gb300.Scene in it.  Imported by tests/, by the smoke check and by bench.py's CPU
baseline leg; never by the product package.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


class PTParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("totalSpp", ctypes.c_int), ("maxDepth", ctypes.c_int),
                ("minDepth", ctypes.c_int), ("baseSeed", ctypes.c_uint32), ("numShadowRays", ctypes.c_int),
                ("enableBsdfDI", ctypes.c_int)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        vp, i, f, u32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_uint32
        L.ora_scene_create.restype = vp
        L.ora_scene_create.argtypes = [i]
        L.ora_scene_destroy.argtypes = [vp]
        L.ora_add_texture.argtypes = [vp, vp, i, i, i, i]
        L.ora_add_material.argtypes = [vp, i, vp, i, f, i, f, f, f, f, f, i]
        L.ora_add_mesh.argtypes = [vp, vp, i, vp, i, vp, vp, i]
        L.ora_add_emitters.argtypes = [vp, i, vp, i, vp, f]
        L.ora_set_envmap.argtypes = [vp, vp, i, i]
        L.ora_set_camera.argtypes = [vp, vp, f]
        L.ora_commit.argtypes = [vp, i, i, ctypes.c_char_p, i]
        L.ora_num_emitters.argtypes = [vp]
        L.ora_bvh_nodes.argtypes = [vp]
        L.ora_render.argtypes = [vp, ctypes.POINTER(PTParams), vp, i, vp, i, i]
        L.ora_render_paths.argtypes = [vp, ctypes.POINTER(PTParams), u32, vp, i, vp, vp, i]
        L.ora_render_pyramid.argtypes = [vp, ctypes.POINTER(PTParams), i, i, vp]
        L.ora_trace.argtypes = [vp, vp, i, vp, i]
        L.ora_trace_brute64.argtypes = [vp, vp, i, vp, vp]
        L.ora_trace_two64.argtypes = [vp, vp, i, vp, vp, i]
        L.ora_material_integrate.argtypes = [vp, i, vp, vp, i, i, vp]
        L.ora_emitter_ray_roundtrip.argtypes = [vp, i, vp, vp, vp]
        L.ora_mesh_shading_normal.argtypes = [vp, i, i, f, f, vp]
        L.ora_ggx_pdf_integrate.argtypes = [f, f, vp, i, vp]
        L.ora_camera_ray.argtypes = [vp, f, f, vp, vp]
        L.ora_material_eval.argtypes = [vp, i, vp, vp, vp, vp, vp, vp]
        L.ora_material_sample.argtypes = [vp, i, vp, vp, f, f, f, vp, vp, vp, vp]
        L.ora_env_radiance.argtypes = [vp, vp, vp]
        L.ora_env_sample.argtypes = [vp, f, f, vp, vp, vp]
        L.ora_env_pdf.argtypes = [vp, vp]
        L.ora_env_pdf.restype = f
        L.ora_rng_hashseed.argtypes = [u32, u32, u32]
        L.ora_rng_hashseed.restype = u32
        L.ora_rng_stream.argtypes = [u32, i, vp]
        L.ora_rng_floats.argtypes = [u32, i, vp]
        L.ora_rng_ints.argtypes = [u32, u32, i, vp, vp]
        L.ora_ggx_D.argtypes = [f, f, vp]
        L.ora_ggx_D.restype = f
        L.ora_ggx_pdf.argtypes = [f, f, vp, vp]
        L.ora_ggx_pdf.restype = f
        L.ora_ggx_sample.argtypes = [f, f, vp, f, f, vp]
        L.ora_world_to_shading.argtypes = [vp, vp, vp]
        L.ora_shading_to_world.argtypes = [vp, vp, vp]
        L.ora_pwc.argtypes = [vp, i, vp, i, vp, vp, vp]
        L.ora_warp_triangle.argtypes = [f, f, vp, vp]
        L.ora_warp_sphere.argtypes = [f, f, vp, vp]
        L.ora_warp_coshemi.argtypes = [f, f, vp, vp, vp]
        L.ora_warp_disc.argtypes = [f, f, vp]
        L.ora_fresnel_dielectric.argtypes = [f, f, f]
        L.ora_fresnel_dielectric.restype = f
        L.ora_emitter_sample.argtypes = [vp, i, f, f, vp]
        L.ora_emitter_radiance.argtypes = [vp, i, vp, vp, vp]
        L.ora_query_emitter.argtypes = [vp, i, i]
        L.ora_adjoint.argtypes = [vp, ctypes.POINTER(PTParams), vp, vp, vp, vp, vp, i]
        L.ora_light_paths.argtypes = [vp, u32, u32, i, i, vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def f32(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    return a if shape is None else a.reshape(shape)


class OracleScene:
    """A scene inside the oracle.  Mirrors seesharp_gb300.Scene.Prepare's realization."""

    def __init__(self, fp64=False):
        self.L = lib()
        self.h = ctypes.c_void_p(self.L.ora_scene_create(int(fp64)))
        self.fp64 = fp64
        self.W = self.H = 0

    def __del__(self):
        try:
            if self.h:
                self.L.ora_scene_destroy(self.h)
                self.h = None
        except Exception:
            pass

    @classmethod
    def from_scene(cls, scene, fp64=False, commit=True):
        """Builds the oracle copy of a seesharp_gb300.Scene (same order of ids as Prepare)."""
        from seesharp_gb300.scene import DiffuseMaterial, GenericMaterial
        o = cls(fp64)
        tex_ids = {}

        def tex(image, border):
            key = (id(image), int(border))
            if key not in tex_ids:
                d = f32(image.data)
                tex_ids[key] = o.L.ora_add_texture(o.h, _p(d), d.shape[1], d.shape[0], d.shape[2], int(border))
            return tex_ids[key]

        def trgb(t):
            return (t.constColor.array(), -1) if t.Image is None else (np.zeros(3, np.float32), tex(t.Image, t.Border))

        def tmono(t):
            return (t.constColor, -1) if t.Image is None else (0.0, tex(t.Image, t.Border))

        mat_ids, mesh_ids = {}, {}
        for m in scene.Meshes:
            mat = m.Material
            if id(mat) not in mat_ids:
                if isinstance(mat, DiffuseMaterial):
                    c, t = trgb(mat.MaterialParameters.BaseColor)
                    c = f32(c)
                    mat_ids[id(mat)] = o.L.ora_add_material(o.h, 0, _p(c), t, 1.0, -1, 0, 1, 0, 0, 1.45, int(mat.MaterialParameters.Transmitter))
                elif isinstance(mat, GenericMaterial):
                    p = mat.MaterialParameters
                    c, t = trgb(p.BaseColor)
                    c = f32(c)
                    r, rt = tmono(p.Roughness)
                    mat_ids[id(mat)] = o.L.ora_add_material(o.h, 1, _p(c), t, r, rt, p.Metallic, p.SpecularTintStrength, p.Anisotropic,
                                                            p.SpecularTransmittance, p.IndexOfRefraction, 0)
                else:
                    raise TypeError(type(mat))
            V = f32(m.Vertices)
            I = np.ascontiguousarray(m.Indices, np.int32)
            N = None if m.ShadingNormals is None else f32(m.ShadingNormals)
            UV = None if m.TextureCoordinates is None else f32(m.TextureCoordinates)
            mesh_ids[id(m)] = o.L.ora_add_mesh(o.h, _p(V), V.shape[0], _p(I), I.size // 3, _p(N), _p(UV), mat_ids[id(mat)])
        for e in scene.Emitters:
            faces = np.array([e.Triangle.FaceIndex], np.int32)
            rad = f32(e.Radiance.array())
            o.L.ora_add_emitters(o.h, mesh_ids[id(e.Mesh)], _p(faces), 1, _p(rad), float(e.exponent))
        if scene.Background is not None:
            d = f32(scene.Background.Image.data)
            o.L.ora_set_envmap(o.h, _p(d), d.shape[1], d.shape[0])
        if scene.Camera is not None:
            m = f32(scene.Camera.WorldToCamera, (16,))
            o.L.ora_set_camera(o.h, _p(m), float(scene.Camera.VerticalFieldOfView))
        o.mesh_ids = mesh_ids
        o.mat_ids = mat_ids
        if commit:
            o.commit(scene.FrameBuffer.Width, scene.FrameBuffer.Height)
        return o

    def commit(self, W, H):
        err = ctypes.create_string_buffer(512)
        rc = self.L.ora_commit(self.h, int(W), int(H), err, 512)
        if rc != 0:
            raise RuntimeError(err.value.decode())
        self.W, self.H = W, H

    @staticmethod
    def params(W, H, spp, maxDepth, minDepth=1, baseSeed=0xC030114, numShadowRays=1, enableBsdfDI=True):
        return PTParams(W, H, spp, maxDepth, minDepth, baseSeed & 0xFFFFFFFF, numShadowRays, int(bool(enableBsdfDI)))

    def render(self, params, nthreads=None, film=None, iter_first=0, iter_count=None):
        """Progressive render with the frame-buffer running mean.  Returns (film, rays, shadow rays)."""
        nthreads = nthreads or os.cpu_count() or 1
        if film is None:
            film = np.zeros((params.height, params.width, 3), np.float32)
        stats = np.zeros(5, np.uint64)
        n = params.totalSpp - iter_first if iter_count is None else iter_count
        self.L.ora_render(self.h, ctypes.byref(params), _p(film), int(nthreads), _p(stats), int(iter_first), int(n))
        self.last_shading_stats = {"NumMaterialEval": int(stats[2]), "NumMaterialSample": int(stats[3]), "NumMaterialPdf": int(stats[4])}
        return film, int(stats[0]), int(stats[1])

    def render_paths(self, params, sample_index, pixels, nthreads=None):
        nthreads = nthreads or os.cpu_count() or 1
        pixels = np.ascontiguousarray(pixels, np.int32)
        rgb = np.zeros((pixels.size, 3), np.float32)
        stats = np.zeros(2, np.uint64)
        self.L.ora_render_paths(self.h, ctypes.byref(params), int(sample_index), _p(pixels), pixels.size, _p(rgb), _p(stats), int(nthreads))
        return rgb, int(stats[0]), int(stats[1])

    def render_pyramid(self, params, iter_first=0, iter_count=None):
        """The raw and MIS-weighted technique pyramids (PathTracer.RenderTechniquePyramid) of
        iterations [iter_first, iter_first + iter_count): float32 (2, 2*maxDepth, H, W, 3); layer
        2(d-1) is "{d}-hit", 2(d-1)+1 "{d}-next-event"."""
        n = params.totalSpp - iter_first if iter_count is None else iter_count
        pyr = np.zeros((2, 2 * params.maxDepth, params.height, params.width, 3), np.float32)
        if self.L.ora_render_pyramid(self.h, ctypes.byref(params), int(iter_first), int(n), _p(pyr)) != 0:
            raise RuntimeError("the technique pyramid is computed in FP32 only")
        return pyr

    def trace(self, rays, any_hit=False):
        rays = f32(rays, (-1, 8))
        hits = np.zeros((rays.shape[0], 4), np.float32)
        self.L.ora_trace(self.h, _p(rays), rays.shape[0], _p(hits), int(any_hit))
        tri = hits[:, 3].copy().view(np.int32)
        return hits[:, 0], hits[:, 1], hits[:, 2], tri

    def trace_brute64(self, org, dirs, tmin=0.0, with_second=False):
        n = org.shape[0]
        rays = np.zeros((n, 7), np.float64)
        rays[:, 0:3] = org
        rays[:, 3:6] = dirs
        rays[:, 6] = tmin
        hits = np.zeros((n, 4), np.float64)
        second = np.zeros(n, np.float64) if with_second else None
        self.L.ora_trace_brute64(self.h, _p(rays), n, _p(hits), _p(second))
        return hits, second

    def trace_two64(self, rays, nthreads=None):
        """FP64 closest hit of FP32 rays (n x 8: org, tmin, dir, tmax) over the oracle's BVH, with the
        distance of the runner-up surface.  Returns hits (n x 4 doubles: t, u, v, global triangle
        id or -1) and the runner-up distances (tmax when there is none)."""
        rays = np.ascontiguousarray(np.asarray(rays, np.float32).reshape(-1, 8), np.float64)
        n = rays.shape[0]
        hits = np.zeros((n, 4), np.float64)
        second = np.zeros(n, np.float64)
        self.L.ora_trace_two64(self.h, _p(rays), n, _p(hits), _p(second), int(nthreads or os.cpu_count() or 1))
        return hits, second

    def material_integrate(self, mat, point, out_dir, mode, n=1_000_000):
        """99% confidence interval of a Monte Carlo integral over directions (the estimator of
        Material_SampleTransform.cs:40-69): mode 0 the albedo with uniform-sphere sampling, 1 the
        albedo with the material's own sampling, 2 the integral of its pdf."""
        pt, od = f32(point, (11,)), f32(out_dir, (3,))
        ci = np.zeros(2, np.float32)
        if self.L.ora_material_integrate(self.h, int(mat), _p(pt), _p(od), int(mode), int(n), _p(ci)) != 0:
            raise ValueError("invalid material or mode")
        return float(ci[0]), float(ci[1])

    def emitter_ray_roundtrip(self, e, prim_pos, prim_dir):
        """Emitter.SampleRay then SampleRayInverse: (posPrimary, dirPrimary, point, direction, pdf, weight)."""
        out = np.zeros(14, np.float32)
        pp, pd = f32(prim_pos, (2,)), f32(prim_dir, (2,))  # kept alive across the call
        if self.L.ora_emitter_ray_roundtrip(self.h, int(e), _p(pp), _p(pd), _p(out)) != 0:
            raise ValueError("no such emitter")
        return out[0:2], out[2:4], out[4:7], out[7:10], float(out[10]), out[11:14]

    def mesh_shading_normal(self, mesh, face, u, v):
        out = np.zeros(3, np.float32)
        if self.L.ora_mesh_shading_normal(self.h, int(mesh), int(face), float(u), float(v), _p(out)) != 0:
            raise ValueError("no such face")
        return out

    def camera_ray(self, fx, fy):
        o = np.zeros(3, np.float32)
        d = np.zeros(3, np.float32)
        self.L.ora_camera_ray(self.h, float(fx), float(fy), _p(o), _p(d))
        return o, d

    def material_eval(self, mat, point, out_dir, in_dir, components=False):
        pt = f32(point, (11,))
        o = f32(out_dir, (3,))
        i = f32(in_dir, (3,))
        val = np.zeros(3, np.float32)
        pdf = np.zeros(2, np.float32)
        comp = np.zeros(13, np.float32)
        self.L.ora_material_eval(self.h, int(mat), _p(pt), _p(o), _p(i), _p(val), _p(pdf), _p(comp))
        return (val, pdf, comp) if components else (val, pdf)

    def material_sample(self, mat, point, out_dir, u, u1, u2, components=False):
        pt = f32(point, (11,))
        o = f32(out_dir, (3,))
        d = np.zeros(3, np.float32)
        pdf = np.zeros(2, np.float32)
        w = np.zeros(3, np.float32)
        comp = np.zeros(13, np.float32)
        self.L.ora_material_sample(self.h, int(mat), _p(pt), _p(o), float(u), float(u1), float(u2), _p(d), _p(pdf), _p(w), _p(comp))
        return (d, pdf, w, comp) if components else (d, pdf, w)

    def env_radiance(self, d):
        d = f32(d, (3,))
        out = np.zeros(3, np.float32)
        self.L.ora_env_radiance(self.h, _p(d), _p(out))
        return out

    def env_sample(self, u1, u2):
        d = np.zeros(3, np.float32)
        pdf = np.zeros(1, np.float32)
        w = np.zeros(3, np.float32)
        self.L.ora_env_sample(self.h, float(u1), float(u2), _p(d), _p(pdf), _p(w))
        return d, float(pdf[0]), w

    def env_pdf(self, d):
        d = f32(d, (3,))
        return float(self.L.ora_env_pdf(self.h, _p(d)))

    def emitter_sample(self, e, u1, u2):
        out = np.zeros(10, np.float32)
        self.L.ora_emitter_sample(self.h, int(e), float(u1), float(u2), _p(out))
        return out

    def emitter_radiance(self, e, point, d):
        pt = f32(point, (11,))
        dd = f32(d, (3,))
        out = np.zeros(3, np.float32)
        self.L.ora_emitter_radiance(self.h, int(e), _p(pt), _p(dd), _p(out))
        return out

    def query_emitter(self, mesh, face):
        return int(self.L.ora_query_emitter(self.h, int(mesh), int(face)))

    def adjoint(self, params, dldi, n_tex, n_mat, n_em, nthreads=None):
        """FP64 path-replay reference gradient (scene must be fp64)."""
        nthreads = nthreads or os.cpu_count() or 1
        d = f32(dldi)
        out = {"textures": np.zeros(max(n_tex, 1)), "materialBaseColor": np.zeros(max(3 * n_mat, 1)),
               "materialRoughness": np.zeros(max(n_mat, 1)), "emitterRadiance": np.zeros(max(3 * n_em, 1))}
        rc = self.L.ora_adjoint(self.h, ctypes.byref(params), _p(d), _p(out["textures"]), _p(out["materialBaseColor"]),
                                _p(out["materialRoughness"]), _p(out["emitterRadiance"]), int(nthreads))
        if rc != 0:
            raise RuntimeError("oracle adjoint needs an fp64 scene")
        out["textures"] = out["textures"][:n_tex]
        out["materialBaseColor"] = out["materialBaseColor"][:3 * n_mat].reshape(-1, 3)
        out["materialRoughness"] = out["materialRoughness"][:n_mat]
        out["emitterRadiance"] = out["emitterRadiance"][:3 * n_em].reshape(-1, 3)
        return out

    def light_paths(self, seed, iteration, max_depth, n):
        """LightPathCache.TraceAllPaths for paths [0, n): (floats (n, maxDepth+1, 16), ints
        (n, maxDepth+1, 4), lengths (n,)) in the layout of sst_trace_light_paths."""
        stride = max_depth + 1
        vf = np.zeros((n, stride, 16), np.float32)
        vi = np.full((n, stride, 4), -1, np.int32)
        lengths = np.zeros(n, np.int32)
        self.L.ora_light_paths(self.h, seed & 0xFFFFFFFF, iteration & 0xFFFFFFFF, int(max_depth), int(n), _p(vf), _p(vi), _p(lengths))
        return vf, vi, lengths

    def num_emitters(self):
        return int(self.L.ora_num_emitters(self.h))


# ---- stateless helpers ----
def rng_hashseed(b, c, s):
    return int(lib().ora_rng_hashseed(b & 0xFFFFFFFF, c & 0xFFFFFFFF, s & 0xFFFFFFFF))


def rng_stream(seed, n):
    out = np.zeros(n, np.uint32)
    lib().ora_rng_stream(seed & 0xFFFFFFFF, n, _p(out))
    return out


def rng_floats(seed, n):
    out = np.zeros(n, np.float32)
    lib().ora_rng_floats(seed & 0xFFFFFFFF, n, _p(out))
    return out


def rng_ints(seed, mx, n):
    out = np.zeros(n, np.uint32)
    st = np.zeros(1, np.uint32)
    lib().ora_rng_ints(seed & 0xFFFFFFFF, mx, n, _p(out), _p(st))
    return out, int(st[0])


def ggx_D(ax, ay, n):
    n = f32(n, (3,))  # a named array: the pointer must outlive the call
    return float(lib().ora_ggx_D(ax, ay, _p(n)))


def ggx_pdf(ax, ay, o, n):
    o, n = f32(o, (3,)), f32(n, (3,))
    return float(lib().ora_ggx_pdf(ax, ay, _p(o), _p(n)))


def ggx_sample(ax, ay, o, u1, u2):
    out = np.zeros(3, np.float32)
    o = f32(o, (3,))
    lib().ora_ggx_sample(ax, ay, _p(o), u1, u2, _p(out))
    return out


def world_to_shading(n, d):
    out = np.zeros(3, np.float32)
    n, d = f32(n, (3,)), f32(d, (3,))
    lib().ora_world_to_shading(_p(n), _p(d), _p(out))
    return out


def shading_to_world(n, d):
    out = np.zeros(3, np.float32)
    n, d = f32(n, (3,)), f32(d, (3,))
    lib().ora_shading_to_world(_p(n), _p(d), _p(out))
    return out


def pwc(weights, us):
    w = f32(weights)
    u = f32(us)
    idx = np.zeros(u.size, np.int32)
    rel = np.zeros(u.size, np.float32)
    prob = np.zeros(w.size, np.float32)
    lib().ora_pwc(_p(w), w.size, _p(u), u.size, _p(idx), _p(rel), _p(prob))
    return idx, rel, prob


def warp_triangle(u1, u2):
    b = np.zeros(2, np.float32)
    i = np.zeros(2, np.float32)
    lib().ora_warp_triangle(u1, u2, _p(b), _p(i))
    return b, i


def warp_sphere(u1, u2):
    d = np.zeros(3, np.float32)
    i = np.zeros(2, np.float32)
    lib().ora_warp_sphere(u1, u2, _p(d), _p(i))
    return d, i


def warp_coshemi(u1, u2):
    d = np.zeros(3, np.float32)
    pdf = np.zeros(1, np.float32)
    i = np.zeros(2, np.float32)
    lib().ora_warp_coshemi(u1, u2, _p(d), _p(pdf), _p(i))
    return d, float(pdf[0]), i


def warp_disc(u1, u2):
    p = np.zeros(2, np.float32)
    lib().ora_warp_disc(u1, u2, _p(p))
    return p


def ggx_pdf_integrate(ax, ay, out_dir, n=1_000_000):
    od = f32(out_dir, (3,))
    ci = np.zeros(2, np.float32)
    lib().ora_ggx_pdf_integrate(float(ax), float(ay), _p(od), int(n), _p(ci))
    return float(ci[0]), float(ci[1])


def fresnel_dielectric(c, ei, et):
    return float(lib().ora_fresnel_dielectric(c, ei, et))
