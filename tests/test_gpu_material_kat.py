"""The reference's statistical sampling checks (SeeSharp.Tests/Core/Shading/Material_SampleTransform.cs:
119-280) on the device: the albedo estimated with the device's own BSDF sampling
(sst_debug_material_sample, then sst_debug_material_eval at the sampled directions) must overlap, at
99% confidence, the oracle's uniform-sphere estimate of the same integral; and the device pdf
integrated over uniform-sphere directions must overlap 1.  Same RNG streams as the reference test:
32 batches of 2^15 samples, batch i seeded RNG(18273912, i, 1313), three numbers per sample (the 2D
primary sample, then the component choice)."""
import ctypes
import math

import numpy as np
import pytest

from oracle import pyoracle as O
from seesharp_gb300 import (DiffuseEmitter, DiffuseMaterial, FrameBuffer, Matrix4x4, Mesh, PerspectiveCamera, RgbColor, Scene, _native)

from test_oracle_kat import SAMPLING_CASES, SAMPLING_HIT, norm, overlap

pytestmark = pytest.mark.gpu

N = 1 << 20


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def _streams():
    u = np.concatenate([O.rng_floats(O.rng_hashseed(18273912, b, 1313), 3 * (N // 32)).reshape(-1, 3) for b in range(32)], 0)
    return u  # columns: primary x, primary y, component choice


def _device_scene(mat):
    sc = Scene()
    m = Mesh([[-10, -10, -2], [10, -10, -2], [10, 10, -2], [-10, 10, -2]], [0, 1, 2, 0, 2, 3])
    m.Material = mat
    sc.Meshes.append(m)
    e = Mesh([[-1, -1, 5], [1, -1, 5], [1, 1, 5]], [0, 1, 2])
    e.Material = DiffuseMaterial()
    sc.Meshes.append(e)
    sc.Emitters.extend(DiffuseEmitter.MakeFromMesh(e, RgbColor.White))
    sc.Camera = PerspectiveCamera(Matrix4x4.CreateLookAt([0, 0, 3], [0, 0, 0], [0, 1, 0]), 40)
    sc.FrameBuffer = FrameBuffer(8, 8)
    sc.Prepare()
    return sc


def _interval(vals):
    """The reference's interval: mean +- 2.576 sqrt((E[v^2] - E[v]^2) / N), skipped samples counting zero."""
    m = float(np.sum(vals, dtype=np.float64)) / N
    v = float(np.sum(np.asarray(vals, np.float64) ** 2)) / N - m * m
    if v <= 0:
        return m, m
    off = math.sqrt(v) / math.sqrt(N)
    return m - 2.576 * off, m + 2.576 * off


def _eval(sc, od, dirs):
    n = dirs.shape[0]
    pts = np.tile(SAMPLING_HIT, (n, 1))
    outs = np.tile(od, (n, 1)).astype(np.float32)
    vals = np.zeros((n, 3), np.float32)
    pdfs = np.zeros((n, 2), np.float32)
    ins = np.ascontiguousarray(dirs, np.float32)
    _native.check(sc.native.lib.sst_debug_material_eval(sc.native.handle, 0, n, _p(pts), _p(outs), _p(ins), _p(vals), _p(pdfs)))
    return vals, pdfs


@pytest.mark.parametrize("name,make,out,kind", SAMPLING_CASES, ids=[c[0] for c in SAMPLING_CASES])
def test_device_material_sample_transform(name, make, out, kind):
    mat = make()
    sc = _device_scene(mat)
    od = norm(out)
    u = _streams()
    if kind == "albedo":
        pts = np.tile(SAMPLING_HIT, (N, 1))
        outs = np.tile(od, (N, 1)).astype(np.float32)
        us = np.ascontiguousarray(u[:, [2, 0, 1]], np.float32)  # (component, direction x, direction y)
        dirs = np.zeros((N, 3), np.float32)
        pdfs = np.zeros((N, 2), np.float32)
        ws = np.zeros((N, 3), np.float32)
        _native.check(sc.native.lib.sst_debug_material_sample(sc.native.handle, 0, N, _p(pts), _p(outs), _p(us), _p(dirs), _p(pdfs), _p(ws)))
        vals, _ = _eval(sc, od, dirs)
        ok = pdfs[:, 0] > 0
        est = np.where(ok, vals.astype(np.float64).mean(axis=1) / np.where(ok, pdfs[:, 0], 1.0), 0.0)
        dev = _interval(est)
        o = O.OracleScene.from_scene(sc, commit=False)
        ref = o.material_integrate(0, SAMPLING_HIT, od, 0)
        assert overlap(dev, ref), (dev, ref)
    else:
        # uniform directions on the sphere from the primary samples (pdf 1 / 4 pi)
        z = 1.0 - 2.0 * u[:, 0].astype(np.float64)
        r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
        phi = 2.0 * math.pi * u[:, 1].astype(np.float64)
        dirs = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1).astype(np.float32)
        _, pdfs = _eval(sc, od, dirs)
        dev = _interval(pdfs[:, 0].astype(np.float64) * (4.0 * math.pi))
        assert overlap(dev, (1.0, 1.0)), dev
