"""Colours, images, textures and the frame buffer.

Mirrors SimpleImageIO's RgbColor/RgbImage/MonochromeImage as SeeSharp uses them, and SeeSharp's
TextureRgb/TextureMono (Images/TextureRgb.cs, Images/TextureMono.cs, Images/ImageTexture.cs) and
FrameBuffer (Images/FrameBuffer.cs).  Pixel data are float32 numpy arrays, row-major, top row
first.
"""
from __future__ import annotations

import enum
import json

import numpy as np


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
        self.layers = {}
        self.PixelVariance = None
        if self.flags & FrameBuffer.Flags.EstimatePixelVariance:
            self.PixelVariance = VarianceLayer()
            self.AddLayer("variance", self.PixelVariance)

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
        for layer in self.layers.values():
            layer.Init(self.Width, self.Height)
            if isinstance(layer, VarianceLayer):
                layer.Average = 0.0

    def WriteToFile(self, filename=None):
        """Writes the image as a PFM (little endian, bottom row first) and the metadata as JSON.

        EXR output is out of scope; PFM is a lossless float format readable by common tools.
        """
        name = filename or self.filename
        if not name:
            raise ValueError("no filename")
        base = name.rsplit(".", 1)[0]
        with open(base + ".pfm", "wb") as f:
            f.write(b"PF\n%d %d\n-1.0\n" % (self.Width, self.Height))
            f.write(np.ascontiguousarray(self.Image.data[::-1]).astype("<f4").tobytes())
        meta = dict(self.MetaData)
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


__all__ = ["RgbColor", "RgbImage", "MonochromeImage", "TextureRgb", "TextureMono", "BorderHandling", "FrameBuffer",
           "mean_rgb", "rel_mse"]
