"""FrameBuffer.WriteToFile (Images/FrameBuffer.cs:312-368): the layered OpenEXR file with the
outlier layers, the per-layer PFM files, and the JSON metadata."""
import json
import os

import numpy as np

from seesharp_gb300 import FrameBuffer, OutlierReplayCache
from seesharp_gb300.images import RgbLayer, VarianceLayer
from seesharp_gb300 import imagefile


def _buffer():
    rng = np.random.default_rng(2)
    fb = FrameBuffer(6, 4, flags=FrameBuffer.Flags.Recommended | FrameBuffer.Flags.EstimatePixelVariance)
    fb.Image.data[:] = rng.random((4, 6, 3), dtype=np.float32)
    fb.AddLayer("albedo", RgbLayer())
    fb.GetLayer("albedo").Image.data[:] = rng.random((4, 6, 3), dtype=np.float32)
    fb.PixelVariance.Image.data[:] = rng.random((4, 6, 1), dtype=np.float32)
    fb.OutlierCache = OutlierReplayCache(6, 4, 2)
    fb.OutlierCache.weight[1, 2] = [1.0, 4.0]
    fb.OutlierCache.iteration[1, 2] = [7, 3]
    fb.Errors = [(10, 0.5, 0.25, 0.2)]
    fb.MetaData["RenderTime"] = 12.5
    return fb


def test_exr_holds_the_image_the_layers_and_the_outlier_iterations(tmp_path):
    fb = _buffer()
    path = str(tmp_path / "img.exr")
    fb.WriteToFile(path)
    ch = imagefile.read_exr_channels(path)
    assert set(ch) == {"R", "G", "B", "albedo.R", "albedo.G", "albedo.B", "variance.Y", "outlier-0.Y", "outlier-1.Y"}
    assert np.array_equal(imagefile.read_exr(path), fb.Image.data)
    assert np.array_equal(ch["albedo.G"], fb.GetLayer("albedo").Image.data[:, :, 1])
    assert np.array_equal(ch["variance.Y"], fb.PixelVariance.Image.data[:, :, 0])
    # descending priority: iteration 3 (weight 4) first
    assert ch["outlier-0.Y"][1, 2] == 3 and ch["outlier-1.Y"][1, 2] == 7
    assert ch["outlier-0.Y"].sum() == 3 and ch["outlier-1.Y"].sum() == 7
    meta = json.load(open(str(tmp_path / "img.json")))
    assert meta["RenderTime"] == 12.5
    assert meta["ErrorMetrics"] == [{"TimeMS": 10, "MSE": 0.5, "RelMSE": 0.25, "RelMSE_Outlier": 0.2}]


def test_other_names_write_one_pfm_per_layer(tmp_path):
    fb = _buffer()
    fb.WriteToFile(str(tmp_path / "img.png"))
    names = sorted(os.listdir(tmp_path))
    assert names == ["img-albedo.pfm", "img-variance.pfm", "img.json", "img.pfm"]
    raw = open(str(tmp_path / "img.pfm"), "rb").read()
    head = b"PF\n6 4\n-1.0\n"
    assert raw.startswith(head)
    img = np.frombuffer(raw[len(head):], "<f4").reshape(4, 6, 3)[::-1]
    assert np.array_equal(img, fb.Image.data)
    mono = open(str(tmp_path / "img-variance.pfm"), "rb").read()
    assert mono.startswith(b"Pf\n6 4\n-1.0\n")
