"""Intersection parity on the benchmark scenes, through the C ABI (sst_trace, sst_occluded).

The reference crosses into Embree for every ray (TinyEmbree Raytracer.Trace / IsOccluded,
Integrators/PathTracer.cs:319,467).  Its only pin on the results is SeeSharp.Tests/Core/
Scene_Assemble.cs:51-63 (t = 10 to 4 decimals), so the referee here is the oracle's FP64 watertight
intersection over its own BVH: on non-degenerate rays the GPU's hit must name the same primitive
exactly and agree in t to a relative 1e-5, and occlusion must agree.

Non-degenerate means: the FP64 hit is at least 1e-4 (in barycentric terms) inside its triangle,
the next surface along the ray is at least a relative 1e-4 farther, and the hit distance is at least
5% of the largest origin coordinate (so that a relative 1e-5 in t is above the FP32 rounding of the
origin and of the vertices).

Rays per scene: camera rays through random film positions and bounce-2 rays spawned from the FP64
primary hits (cosine-distributed about the face normal on the incoming side, plus uniform
directions on the other side, origins offset by the hit's error offset as SpawnRay does), and
shadow segments from those origins to random points on the emitters (IsOccluded's form: an
unnormalised direction and tmax = 1 - 1e-5).
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from seesharp_gb300 import _native, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[2, 4, 8], ids=["bvh2", "bvh4", "bvh8"])
def width(request):
    ctx = _native.default_context()
    base = _native.get_tuning(ctx)
    _native.set_tuning(ctx, traceBvhWidth=request.param)
    yield request.param
    _native.set_tuning(ctx, **base)


def _mesh_offsets(sc):
    off, n = [], 0
    for m in sc.Meshes:
        off.append(n)
        n += np.asarray(m.Indices).size // 3
    return np.array(off + [n], np.int64)


def _tri_table(sc):
    V = []
    for m in sc.Meshes:
        v = np.asarray(m.Vertices, np.float64).reshape(-1, 3)
        V.append(v[np.asarray(m.Indices, np.int64).reshape(-1, 3)])
    return np.concatenate(V, 0)  # (triangles, 3 corners, 3)


def _error_offset(tri, u, v):
    # Mesh.ComputeErrorOffset (Geometry/Mesh.cs:50-60), u and v weighting the 2nd and 3rd vertex
    e = np.abs(u[:, None] * tri[:, 1]) + np.abs(v[:, None] * tri[:, 2]) + np.abs((1 - u - v)[:, None] * tri[:, 0])
    return np.linalg.norm(e, axis=1) * 32.0 * 1.19209e-07


def _rays_for(sc, o, rng, n_cam=2000):
    W, H = sc.FrameBuffer.Width, sc.FrameBuffer.Height
    film = rng.uniform(0, 1, size=(n_cam, 2)) * [W, H]
    cam = np.zeros((n_cam, 8), np.float32)
    for i in range(n_cam):
        org, d = o.camera_ray(*film[i])
        cam[i, 0:3], cam[i, 4:7] = org, d
    cam[:, 7] = np.inf
    hits, _ = o.trace_two64(cam)
    tris = _tri_table(sc)
    sel = hits[:, 3] >= 0
    h = hits[sel]
    g = h[:, 3].astype(np.int64)
    tri = tris[g]
    u, v = h[:, 1], h[:, 2]
    pos = (1 - u - v)[:, None] * tri[:, 0] + u[:, None] * tri[:, 1] + v[:, None] * tri[:, 2]
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    eps = _error_offset(tri, u, v)
    din = cam[sel, 4:7].astype(np.float64)
    side = -np.sign(np.sum(din * nrm, axis=1))  # the incoming side
    side[side == 0] = 1
    m = pos.shape[0]
    # bounce-2 directions: cosine lobe about the normal on the incoming side for 3/4, uniform on the
    # other side (transmission) for the rest
    z = rng.normal(size=(m, 3))
    z /= np.linalg.norm(z, axis=1, keepdims=True)
    d2 = nrm * side[:, None] + z
    refl = rng.random(m) < 0.75
    d2[~refl] = z[~refl] * np.where(np.sum(z[~refl] * nrm[~refl], axis=1) * side[~refl] > 0, -1, 1)[:, None]
    d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
    s = np.where(np.sum(d2 * nrm, axis=1) < 0, -1.0, 1.0)
    org2 = pos + (s * eps)[:, None] * nrm
    sec = np.zeros((m, 8), np.float32)
    sec[:, 0:3], sec[:, 4:7], sec[:, 7] = org2, d2, np.inf
    # shadow segments toward random points on the emitters (or random scene points without any)
    em = [e for e in sc.Emitters]
    if em:
        pick = rng.integers(0, len(em), size=m)
        r1, r2 = rng.random(m), rng.random(m)
        sq = np.sqrt(r1)
        b1, b2 = 1 - sq, r2 * sq
        lp = np.zeros((m, 3))
        for k in range(m):
            e = em[pick[k]]
            V = np.asarray(e.Mesh.Vertices, np.float64).reshape(-1, 3)
            I = np.asarray(e.Mesh.Indices, np.int64).reshape(-1, 3)[e.Triangle.FaceIndex]
            lp[k] = (1 - b1[k] - b2[k]) * V[I[0]] + b1[k] * V[I[1]] + b2[k] * V[I[2]]
    else:
        lp = pos[rng.permutation(m)]
    dd = lp - pos
    s3 = np.where(np.sum(dd * nrm, axis=1) < 0, -1.0, 1.0)
    org3 = pos + (s3 * eps)[:, None] * nrm
    shadow = np.zeros((m, 8), np.float32)
    shadow[:, 0:3], shadow[:, 4:7], shadow[:, 7] = org3, (lp - org3), 1.0 - 1e-5
    return cam, sec, shadow


def _check_closest(sc, o, rays, offsets, label):
    hits = sc.native.trace(rays).view(np.float32)
    mesh_id = hits[:, 4].view(np.int32)
    prim = hits[:, 3].view(np.int32)
    ref, second = o.trace_two64(rays)
    checked = 0
    for i in range(rays.shape[0]):
        rt, ru, rv, rg = ref[i]
        rg = int(rg)
        if rg < 0:
            if mesh_id[i] >= 0:
                # a GPU hit where FP64 finds none must be an edge graze
                gu, gv = hits[i, 1], hits[i, 2]
                assert min(gu, gv, 1 - gu - gv) < 1e-4, (label, i, mesh_id[i], prim[i])
            else:
                checked += 1
            continue
        w = 1 - ru - rv
        if min(ru, rv, w) < 1e-4 or (second[i] - rt) < 1e-4 * rt or rt < 0.05 * max(np.abs(rays[i, 0:3]).max(), 1.0):
            continue
        mesh = int(np.searchsorted(offsets, rg, side="right") - 1)
        assert mesh_id[i] == mesh and prim[i] == rg - offsets[mesh], (label, i, mesh_id[i], prim[i], mesh, rg - offsets[mesh])
        assert abs(hits[i, 0] - rt) <= 1e-5 * rt, (label, i, hits[i, 0], rt)
        checked += 1
    return checked


def _occlusion_reference(o, rays, tris):
    """FP64 occlusion of each segment and whether the answer is robust to FP32 rounding: the first
    surface along the segment's line is farther from the segment's end than the FP32 resolution of
    its t (16 ulps of the segment's coordinates over the segment's length, divided by the cosine
    between the segment and the surface normal, since a grazing hit's t moves with every ulp of the
    other coordinates; at least a relative 1e-6), and an occluder in front of the end is at least
    1e-4 (in barycentric terms) inside its triangle."""
    full = rays.copy()
    full[:, 7] = np.inf
    ref, _ = o.trace_two64(full)
    org, d = rays[:, 0:3].astype(np.float64), rays[:, 4:7].astype(np.float64)
    tmax = rays[:, 7].astype(np.float64)
    span = np.maximum(np.maximum(np.abs(org).max(axis=1), np.abs(org + d).max(axis=1)), 1.0)
    dl = np.linalg.norm(d, axis=1)
    tri = tris[np.maximum(ref[:, 3], 0).astype(np.int64)]
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    cos = np.abs(np.sum(nrm * d, axis=1)) / np.maximum(np.linalg.norm(nrm, axis=1) * dl, 1e-300)
    res = np.maximum(16 * 1.2e-7 * span / dl / np.maximum(cos, 1e-9), 1e-6 * tmax)
    hit = ref[:, 3] >= 0
    rt, ru, rv = ref[:, 0], ref[:, 1], ref[:, 2]
    want = hit & (rt < tmax)
    decisive = ~hit | (np.abs(rt - tmax) > res)
    decisive &= ~(want & (np.minimum(np.minimum(ru, rv), 1 - ru - rv) < 1e-4))
    return want, decisive


def _check_occluded(sc, o, rays, label):
    occ = sc.native.occluded(rays) != 0
    want, decisive = _occlusion_reference(o, rays, _tri_table(sc))
    bad = np.nonzero(decisive & (occ != want))[0]
    assert bad.size == 0, (label, bad[:8], occ[bad[:8]], want[bad[:8]])
    return int(decisive.sum())


def _run(sc, seed, min_frac=0.5):
    sc.Prepare()
    o = O.OracleScene.from_scene(sc, fp64=True)
    rng = np.random.default_rng(seed)
    cam, sec, shadow = _rays_for(sc, o, rng)
    off = _mesh_offsets(sc)
    n_cam = _check_closest(sc, o, cam, off, "camera")
    n_sec = _check_closest(sc, o, sec, off, "bounce-2")
    n_occ = _check_occluded(sc, o, shadow, "shadow")
    assert cam.shape[0] + sec.shape[0] + shadow.shape[0] >= 4000
    assert n_cam >= min_frac * cam.shape[0], n_cam
    assert n_sec >= min_frac * sec.shape[0], n_sec
    assert n_occ >= min_frac * shadow.shape[0], n_occ
    return n_cam, n_sec, n_occ


def test_intersection_cornell_box(width):
    """The 36-triangle Cornell-box configuration (256 x 256)."""
    _run(workloads.cornell_box(256, 256), 1)


def test_intersection_sphere_field_1m(width):
    """The 1M-triangle benchmark scene: 200 displaced icospheres, ground, 50 emitters."""
    sc = workloads.sphere_field(200, 1024, 1024)
    _run(sc, 2)


def test_intersection_large_combined_slice(width):
    """A ~1M-triangle slice of the large combined generator: 150 icospheres over a 256^2-quad
    terrain with 100 emitters (the full job is 2000 icospheres over 1024^2 quads)."""
    sc, _, _, cams = workloads.large_combined(480, 270, num_spheres=150, terrain_quads=256, tex_res=64, num_lights=100, views=2)
    _run(sc, 3)
