"""Colours, images, textures and the frame buffer.

Mirrors SimpleImageIO's RgbColor/RgbImage/MonochromeImage as SeeSharp uses them, and SeeSharp's
TextureRgb/TextureMono (Images/TextureRgb.cs, Images/TextureMono.cs, Images/ImageTexture.cs) and
FrameBuffer (Images/FrameBuffer.cs).  Pixel data are float32 numpy arrays, row-major, top row
first.
"""
from __future__ import annotations

import enum
import json
import os
from collections import namedtuple

import numpy as np

# Images/Pixel.cs: integer pixel coordinates, column from the left, row from the top
Pixel = namedtuple("Pixel", "Col Row")


class RgbColor:
    """Immutable RGB triple in float32 (SimpleImageIO.RgbColor)."""

    __slots__ = ("_v",)

    def __init__(self, r, g=None, b=None):
        if g is None:
            if isinstance(r, RgbColor):
                self._v = r._v.copy()
                return
            arr = np.asarray(r, dtype=np.float32)
            if arr.ndim == 0:
                self._v = np.array([arr, arr, arr], dtype=np.float32)
            else:
                self._v = arr.reshape(3).astype(np.float32)
        else:
            self._v = np.array([r, g, b], dtype=np.float32)

    R = property(lambda s: float(s._v[0]))
    G = property(lambda s: float(s._v[1]))
    B = property(lambda s: float(s._v[2]))

    @property
    def Average(self):
        return float((self._v[0] + self._v[1] + self._v[2]) / np.float32(3))

    @property
    def Luminance(self):
        v = self._v
        return float(np.float32(0.2126) * v[0] + np.float32(0.7152) * v[1] + np.float32(0.0722) * v[2])

    def array(self):
        return self._v.copy()

    def __iter__(self):
        return iter(float(x) for x in self._v)

    def __mul__(self, o):
        return RgbColor(self._v * (o._v if isinstance(o, RgbColor) else np.float32(o)))

    __rmul__ = __mul__

    def __truediv__(self, o):
        return RgbColor(self._v / (o._v if isinstance(o, RgbColor) else np.float32(o)))

    def __add__(self, o):
        return RgbColor(self._v + o._v)

    def __sub__(self, o):
        return RgbColor(self._v - o._v)

    def __eq__(self, o):
        return isinstance(o, RgbColor) and bool(np.all(self._v == o._v))

    def __hash__(self):
        return hash(tuple(self._v.tolist()))

    def __repr__(self):
        return f"RgbColor({self._v[0]:g}, {self._v[1]:g}, {self._v[2]:g})"


RgbColor.White = RgbColor(1.0, 1.0, 1.0)
RgbColor.Black = RgbColor(0.0, 0.0, 0.0)


class Image:
    """Base of RgbImage / MonochromeImage: float32 data of shape (height, width, channels)."""

    channels = 1

    def __init__(self, width, height=None, data=None):
        if isinstance(width, np.ndarray):
            data = width
        if data is not None:
            data = np.ascontiguousarray(data, dtype=np.float32)
            if data.ndim == 2:
                data = data[:, :, None]
            if data.shape[2] != self.channels:
                raise ValueError(f"expected {self.channels} channels, got {data.shape[2]}")
            self.data = data
        else:
            self.data = np.zeros((int(height), int(width), self.channels), dtype=np.float32)

    Width = property(lambda s: s.data.shape[1])
    Height = property(lambda s: s.data.shape[0])


class RgbImage(Image):
    channels = 3

    def GetPixel(self, col, row):
        return RgbColor(self.data[row, col])

    def SetPixel(self, col, row, color):
        self.data[row, col] = RgbColor(color).array()

    def AtomicAdd(self, col, row, color):
        self.data[row, col] += RgbColor(color).array()

    def Scale(self, s):
        self.data *= np.float32(s)


class MonochromeImage(Image):
    channels = 1

    def GetPixel(self, col, row):
        return float(self.data[row, col, 0])


class BorderHandling(enum.IntEnum):
    """ImageTexture.BorderHandling (Images/ImageTexture.cs:8-22)."""
    Repeat = 0
    Clamp = 1


class ImageTexture:
    Border = BorderHandling.Repeat
    Image = None

    @property
    def IsConstant(self):
        return self.Image is None


class TextureRgb(ImageTexture):
    """Constant colour or RGB image (Images/TextureRgb.cs:6-37)."""

    def __init__(self, value):
        self.Border = BorderHandling.Repeat
        if isinstance(value, RgbImage):
            self.Image = value
            self.constColor = None
        else:
            self.Image = None
            self.constColor = RgbColor(value)


class TextureMono(ImageTexture):
    """Constant value or monochrome image (Images/TextureMono.cs:6-40)."""

    def __init__(self, value):
        self.Border = BorderHandling.Repeat
        if isinstance(value, MonochromeImage):
            self.Image = value
            self.constColor = None
        else:
            self.Image = None
            self.constColor = float(np.float32(value))


class Layer:
    """Images/Layer.cs: an auxiliary frame-buffer image, a running mean over the iterations."""

    def __init__(self):
        self.Image = None

    def Init(self, width, height):
        raise NotImplementedError


class RgbLayer(Layer):
    """Images/RgbLayer.cs: an RGB running mean (the denoiser's "albedo" and "normal" features)."""

    def Init(self, width, height):
        self.Image = RgbImage(width, height)


class VarianceLayer(Layer):
    """Images/VarianceLayer.cs: the relative pixel variance image (MonochromeImage) and its
    average, filled by the GPU film fold when the frame buffer has EstimatePixelVariance.  The
    running means of the iteration values and of their squares are kept for resumed renders."""

    def __init__(self):
        super().__init__()
        self.Average = 0.0
        self.state = None

    def Init(self, width, height):
        self.Image = MonochromeImage(width, height)
        self.state = np.zeros((2, height, width), np.float32)


class OutlierReplayCache:
    """Integrators/Util/OutlierReplayCache.cs: per pixel the n samples with the largest channel
    average, with the (0-based) iteration that produced them, so that a path can be replayed from
    its seed.  The heaps are kept by the GPU film fold in the array order of .NET's PriorityQueue
    (a 4-ary min-heap); GetPixelOutlier returns that order, as PriorityQueue.UnorderedItems does.
    Only the sample's channel average (the priority) is kept, not its RGB weight."""

    PathReplayInfo = namedtuple("PathReplayInfo", "Iteration")
    Item = namedtuple("Item", "Element Priority")

    class PixelOutliers:
        def __init__(self, items):
            self.UnorderedItems = items
            self.Count = len(items)

    def __init__(self, width, height, n):
        self.width, self.nMax = int(width), int(n)
        self.weight = np.zeros((int(height), self.width, self.nMax), np.float32)
        self.iteration = np.full((int(height), self.width, self.nMax), -1, np.int32)

    def GetPixelOutlier(self, pixel):
        col, row = pixel
        return OutlierReplayCache.PixelOutliers([OutlierReplayCache.Item(OutlierReplayCache.PathReplayInfo(int(i)), float(w))
                                                 for w, i in zip(self.weight[row, col], self.iteration[row, col]) if i >= 0])

    def outlier_layers(self):
        """FrameBuffer.WriteToFile's "outlier-i" images (FrameBuffer.cs:321-335): per pixel the
        iterations ordered by descending priority (a stable sort of the heap array), 0 where a
        pixel has fewer entries."""
        h, w, n = self.weight.shape
        key = np.where(self.iteration >= 0, self.weight, -np.inf)
        order = np.argsort(-key, axis=2, kind="stable")
        its = np.take_along_axis(self.iteration, order, axis=2)
        its = np.where(its >= 0, its, 0).astype(np.float32)
        return [its[:, :, i] for i in range(n)]


class FrameBuffer:
    """Progressive film with a running mean over iterations (Images/FrameBuffer.cs).

    Image holds the mean of all finished iterations.  Rendering happens on the GPU; this object
    carries the host copy, the iteration count and the metadata the integrator writes.
    """

    class Flags(enum.IntFlag):
        # Images/FrameBuffer.cs:100-133
        None_ = 0
        WriteIntermediate = 1
        WriteContinously = 2
        SendToTev = 4
        EstimatePixelVariance = 8
        IgnoreNanAndInf = 16
        WriteExponentially = 32
        Recommended = 16

    def __init__(self, width, height, filename="", flags=None):
        self.Width = int(width)
        self.Height = int(height)
        self.filename = filename
        self.flags = FrameBuffer.Flags.Recommended if flags is None else FrameBuffer.Flags(flags)
        self.Image = RgbImage(self.Width, self.Height)
        self.CurIteration = 0
        self.MetaData = {}
        self.NaNWarnings = []
        self.ReferenceImage = None   # RgbImage: per-iteration error metrics are recorded in Errors
        self.Errors = []             # (TimeMS, MSE, RelMSE, RelMSE_Outlier) per iteration
        self.NumOutliersToTrack = 4  # FrameBuffer.cs:36; 0..8 on the GPU
        self.OutlierCache = None     # created with the first iteration (FrameBuffer.Initialize, :229)
        self.layers = {}
        self.PixelVariance = None
        if self.flags & FrameBuffer.Flags.EstimatePixelVariance:
            self.PixelVariance = VarianceLayer()
            self.AddLayer("variance", self.PixelVariance)

    @property
    def Basename(self):
        """FrameBuffer.Basename (FrameBuffer.cs:79-87): the image file's path without its extension."""
        if not self.filename:
            return ""
        return os.path.join(os.path.dirname(self.filename), os.path.splitext(os.path.basename(self.filename))[0])

    def AddLayer(self, name, layer):
        """FrameBuffer.AddLayer (FrameBuffer.cs:60): the layer is initialised to the buffer's size."""
        layer.Init(self.Width, self.Height)
        self.layers[name] = layer

    def GetLayer(self, name):
        return self.layers[name]

    @property
    def IgnoreNanAndInf(self):
        return bool(self.flags & FrameBuffer.Flags.IgnoreNanAndInf)

    def Reset(self):
        """FrameBuffer.Reset (FrameBuffer.cs:296-299) plus clearing the image and the layers."""
        self.CurIteration = 0
        self.Image = RgbImage(self.Width, self.Height)
        self.Errors = []
        self.OutlierCache = None
        for layer in self.layers.values():
            layer.Init(self.Width, self.Height)
            if isinstance(layer, VarianceLayer):
                layer.Average = 0.0

    def WriteToFile(self, filename=None):
        """FrameBuffer.WriteToFile (FrameBuffer.cs:312-368).  An ".exr" name gets one layered
        OpenEXR file: the image as R, G, B, every layer as "<name>.R/G/B" (RGB) or "<name>.Y"
        (monochrome), and the outlier cache's "outlier-i" images.  Any other name gets a PFM of the
        image (little endian, bottom row first) and one PFM per layer, "<base>-<layer>.pfm".  The
        metadata (with the error metrics and NaN warnings) goes to "<base>.json"."""
        from . import imagefile
        name = filename or self.filename
        if not name:
            raise ValueError("no filename")
        base, ext = os.path.splitext(name)
        images = [(n, layer.Image) for n, layer in self.layers.items() if layer.Image is not None]
        if ext.lower() == ".exr":
            ch = {}
            for n, img in images + [(None, self.Image)]:
                d = np.asarray(img.data, np.float32)
                prefix = "" if n is None else n + "."
                if d.ndim == 3 and d.shape[2] == 3:
                    for c, k in zip("RGB", range(3)):
                        ch[prefix + c] = d[:, :, k]
                else:
                    ch[prefix + "Y"] = d.reshape(self.Height, self.Width)
            if self.OutlierCache is not None:
                for i, img in enumerate(self.OutlierCache.outlier_layers()):
                    ch[f"outlier-{i}.Y"] = img
            imagefile.write_exr(name, ch)
        else:
            def pfm(path, d):
                d = np.asarray(d, np.float32)
                rgb = d.ndim == 3 and d.shape[2] == 3
                with open(path, "wb") as f:
                    f.write(b"%s\n%d %d\n-1.0\n" % (b"PF" if rgb else b"Pf", self.Width, self.Height))
                    f.write(np.ascontiguousarray(d.reshape(self.Height, self.Width, -1)[::-1]).astype("<f4").tobytes())
            pfm(base + ".pfm", self.Image.data)
            for n, img in images:
                pfm(f"{base}-{n}.pfm", img.data)
        meta = dict(self.MetaData)
        if self.Errors:
            meta["ErrorMetrics"] = [{"TimeMS": t, "MSE": a, "RelMSE": b, "RelMSE_Outlier": c} for (t, a, b, c) in self.Errors]
        meta["NaNWarnings"] = [{"Pixel": {"Col": c, "Row": r}, "Iteration": it} for (c, r, it) in self.NaNWarnings]
        with open(base + ".json", "w") as f:
            json.dump(meta, f, default=lambda o: o.__dict__ if hasattr(o, "__dict__") else str(o))


def mean_rgb(image_data):
    """Validator.ValidateImages' image mean (SeeSharp.Validation/Validator.cs:10-22)."""
    d = np.asarray(image_data, dtype=np.float64)
    return float(d.sum() / (3 * d.shape[0] * d.shape[1]))


def rel_mse(image, reference, eps=1e-2):
    """Relative MSE: mean over pixels and channels of (x - r)^2 / (r^2 + eps).

    SimpleImageIO's Metrics.RelMSE is not vendored; this is the definition used here.
    """
    x = np.asarray(image, dtype=np.float64)
    r = np.asarray(reference, dtype=np.float64)
    return float(np.mean((x - r) ** 2 / (r * r + eps)))


def rel_mse_outlier_rejection(image, reference, percentage=0.1, eps=1e-2):
    """Relative MSE without the worst pixels (SimpleImageIO's Metrics.RelMSE_OutlierRejection, not
    vendored; this is the definition used here and by the GPU error metrics): each pixel's error is
    its mean over the channels of (x - r)^2 / (r^2 + eps); the largest floor(pixels * percentage /
    100) are dropped and the rest averaged."""
    x = np.asarray(image, dtype=np.float32)
    r = np.asarray(reference, dtype=np.float32)
    d = (x - r).astype(np.float64)
    r64 = r.astype(np.float64)
    e = (d * d / (r64 * r64 + eps)).sum(axis=-1) / 3.0
    e = np.sort(e.astype(np.float32).ravel())
    k = int(e.size * percentage / 100)
    return float(np.sum(e[:e.size - k], dtype=np.float64) / (e.size - k))


__all__ = ["RgbColor", "RgbImage", "MonochromeImage", "TextureRgb", "TextureMono", "BorderHandling", "FrameBuffer",
           "OutlierReplayCache", "Pixel", "mean_rgb", "rel_mse", "rel_mse_outlier_rejection"]
