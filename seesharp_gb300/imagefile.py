"""Image files for scene loading: OpenEXR and PNG readers (stand-ins for SimpleImageIO 1.8.3,
which SeeSharp's RgbImage(filename) / TextureRgb(filename) use and which is not vendored).

Both readers are written from the published file-format specifications:

* OpenEXR: single-part scan-line files with HALF or FLOAT channels, compressed NONE, ZIPS or ZIP
  (zlib, then the byte predictor and the even/odd byte split of the format undone).  The R, G,
  B channels are returned (a lone Y channel is replicated); A is dropped.
* PNG: non-interlaced, bit depth 8 or 16, grey / grey+alpha / RGB / RGBA / palette, all five
  scan-line filters.  8- and 16-bit values are decoded to linear RGB with the sRGB transfer
  function, SimpleImageIO's documented treatment of LDR files.

Images come back as float32 arrays (height, width, 3), first row at the top, as RgbImage holds them.
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np


# ---------------------------------------------------------------------------------------------
# OpenEXR
# ---------------------------------------------------------------------------------------------
_EXR_MAGIC = 20000630
_EXR_LINES = {0: 1, 2: 1, 3: 16}   # lines per chunk for NONE, ZIPS, ZIP
_EXR_TYPES = {1: np.float16, 2: np.float32}


def _exr_header(b):
    magic, version = struct.unpack_from("<ii", b, 0)
    if magic != _EXR_MAGIC:
        raise ValueError("not an OpenEXR file")
    if version & 0x200 or version & 0x800 or version & 0x1000:
        raise NotImplementedError("tiled, deep or multi-part OpenEXR files are not supported")
    p, attrs = 8, {}
    while True:
        e = b.index(b"\0", p)
        name = b[p:e].decode()
        p = e + 1
        if not name:
            return attrs, p
        e = b.index(b"\0", p)
        typ = b[p:e].decode()
        p = e + 1
        (size,) = struct.unpack_from("<i", b, p)
        p += 4
        attrs[name] = (typ, b[p:p + size])
        p += size


def _exr_channels(raw):
    out, p = [], 0
    while raw[p] != 0:
        e = raw.index(b"\0", p)
        name = raw[p:e].decode()
        ptype, _plinear, xs, ys = struct.unpack_from("<iB3xii", raw, e + 1)
        if xs != 1 or ys != 1:
            raise NotImplementedError("sub-sampled OpenEXR channels are not supported")
        out.append((name, ptype))
        p = e + 1 + 16
    return out


def _exr_unzip(data, expected):
    t = np.frombuffer(zlib.decompress(data), np.uint8)
    if t.size != expected:
        raise ValueError("corrupt OpenEXR ZIP block")
    # predictor: each byte was stored as the difference to its predecessor plus 128
    d = ((np.cumsum(t.astype(np.int64) - 128) + 128) & 0xFF).astype(np.uint8)
    # the bytes were split into even and odd positions
    half = (t.size + 1) // 2
    out = np.empty(t.size, np.uint8)
    out[0::2] = d[:half]
    out[1::2] = d[half:]
    return out.tobytes()


def read_exr_channels(path):
    """Every channel of a scan-line OpenEXR file: {name: float32 (height, width)}."""
    with open(path, "rb") as f:
        b = f.read()
    attrs, p = _exr_header(b)
    comp = attrs["compression"][1][0]
    if comp not in _EXR_LINES:
        raise NotImplementedError(f"OpenEXR compression {comp} is not supported (NONE, ZIPS and ZIP are)")
    xmin, ymin, xmax, ymax = struct.unpack("<4i", attrs["dataWindow"][1])
    w, h = xmax - xmin + 1, ymax - ymin + 1
    chans = _exr_channels(attrs["channels"][1])
    for _, t in chans:
        if t not in _EXR_TYPES:
            raise NotImplementedError("UINT OpenEXR channels are not supported")
    lines = _EXR_LINES[comp]
    nchunks = (h + lines - 1) // lines
    offsets = struct.unpack_from(f"<{nchunks}Q", b, p)
    planes = {name: np.zeros((h, w), np.float32) for name, _ in chans}
    for off in offsets:
        y, size = struct.unpack_from("<ii", b, off)
        data = b[off + 8: off + 8 + size]
        y0 = y - ymin
        n = min(lines, h - y0)
        bytes_per_line = sum(w * np.dtype(_EXR_TYPES[t]).itemsize for _, t in chans)
        expected = n * bytes_per_line
        if comp != 0 and size < expected:
            data = _exr_unzip(data, expected)
        q = 0
        for r in range(n):
            for name, t in chans:   # channels are stored in the header's (alphabetical) order
                dt = np.dtype(_EXR_TYPES[t]).newbyteorder("<")
                cnt = w * dt.itemsize
                planes[name][y0 + r] = np.frombuffer(data, dt, count=w, offset=q).astype(np.float32)
                q += cnt
    return planes


def read_exr(path):
    planes = read_exr_channels(path)
    if all(c in planes for c in "RGB"):
        rgb = np.stack([planes["R"], planes["G"], planes["B"]], -1)
    elif "Y" in planes:
        rgb = np.repeat(planes["Y"][:, :, None], 3, axis=2)
    else:
        raise ValueError("OpenEXR file has neither R, G, B nor Y channels")
    return np.ascontiguousarray(rgb, np.float32)


def _attr(name, typ, payload):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(payload)) + payload


def write_exr(path, channels):
    """A single-part scan-line OpenEXR file, uncompressed, FLOAT channels.  channels: {name: (height,
    width) array}; layer channels are named "layer.R" and so on, the main image "R", "G", "B".
    Channels are stored in the alphabetical order the format requires."""
    names = sorted(channels)
    if not names:
        raise ValueError("no channels")
    h, w = np.shape(channels[names[0]])
    planes = []
    for n in names:
        a = np.asarray(channels[n], np.float32)
        if a.shape != (h, w):
            raise ValueError(f"channel {n} has shape {a.shape}, expected {(h, w)}")
        planes.append(a.astype("<f4"))
    chlist = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", 2, 0, 1, 1) for n in names) + b"\0"
    header = struct.pack("<ii", _EXR_MAGIC, 2)
    header += _attr("channels", "chlist", chlist)
    header += _attr("compression", "compression", b"\0")
    header += _attr("dataWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1))
    header += _attr("displayWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1))
    header += _attr("lineOrder", "lineOrder", b"\0")
    header += _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
    header += _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
    header += _attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
    header += b"\0"
    line_bytes = 4 * w * len(names)
    start = len(header) + 8 * h
    offsets = struct.pack(f"<{h}Q", *[start + y * (8 + line_bytes) for y in range(h)])
    with open(path, "wb") as f:
        f.write(header)
        f.write(offsets)
        for y in range(h):
            f.write(struct.pack("<ii", y, line_bytes))
            for pl in planes:
                f.write(pl[y].tobytes())


# ---------------------------------------------------------------------------------------------
# PNG
# ---------------------------------------------------------------------------------------------
_PNG_SIG = b"\x89PNG\r\n\x1a\n"
_PNG_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter(raw, h, stride, bpp):
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    p = 0
    for y in range(h):
        ft = raw[p]
        line = np.frombuffer(raw, np.uint8, count=stride, offset=p + 1).astype(np.int32)
        p += stride + 1
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 0xFF
        elif ft == 1:
            cur = np.empty_like(line)
            for k in range(bpp):   # running sum per byte lane
                cur[k::bpp] = np.cumsum(line[k::bpp]) & 0xFF
        elif ft in (3, 4):
            cur = line.copy()
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                if ft == 3:
                    pred = (a + prev[x]) >> 1
                else:
                    pred = _paeth(a, int(prev[x]), int(prev[x - bpp]) if x >= bpp else 0)
                cur[x] = (cur[x] + pred) & 0xFF
        else:
            raise ValueError(f"corrupt PNG: filter type {ft}")
        out[y] = cur
        prev = cur
    return out


def srgb_to_linear(v):
    v = np.asarray(v, np.float64)
    return np.where(v <= 0.04045, v / 12.92, ((v + 0.055) / 1.055) ** 2.4)


def read_png(path):
    with open(path, "rb") as f:
        b = f.read()
    if b[:8] != _PNG_SIG:
        raise ValueError("not a PNG file")
    p, idat, palette = 8, [], None
    w = h = depth = ctype = interlace = None
    while p < len(b):
        length, typ = struct.unpack_from(">I4s", b, p)
        body = b[p + 8: p + 8 + length]
        p += 12 + length
        if typ == b"IHDR":
            w, h, depth, ctype, _comp, _filt, interlace = struct.unpack(">IIBBBBB", body)
        elif typ == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif typ == b"IDAT":
            idat.append(body)
        elif typ == b"IEND":
            break
    if interlace:
        raise NotImplementedError("interlaced PNG files are not supported")
    if depth not in (8, 16) or ctype not in _PNG_CHANNELS:
        raise NotImplementedError(f"PNG bit depth {depth} / colour type {ctype} is not supported")
    ch = _PNG_CHANNELS[ctype]
    bpp = ch * depth // 8
    raw = zlib.decompress(b"".join(idat))
    px = _unfilter(raw, h, w * bpp, bpp)
    if depth == 16:
        vals = px.reshape(h, w * ch, 2).astype(np.uint32)
        vals = ((vals[..., 0] << 8) | vals[..., 1]).reshape(h, w, ch) / 65535.0
    else:
        vals = px.reshape(h, w, ch)
        if ctype == 3:
            vals = palette[vals[..., 0]].astype(np.float64) / 255.0
            ch = 3
        else:
            vals = vals / 255.0
    if ch in (1, 2):
        rgb = np.repeat(vals[..., :1], 3, axis=2)
    else:
        rgb = vals[..., :3]
    return np.ascontiguousarray(srgb_to_linear(rgb), np.float32)


def read_image(path):
    """RGB float32 (height, width, 3) from an .exr or .png file."""
    ext = os.path.splitext(path)[1].lower()
    if ext == ".exr":
        return read_exr(path)
    if ext == ".png":
        return read_png(path)
    raise NotImplementedError(f"image format '{ext}' is not supported (.exr and .png are)")
