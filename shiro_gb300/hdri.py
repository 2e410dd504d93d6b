"""High-dynamic-range environment images from disk, without OpenImageIO.

The reference loads a dome light's image with OpenImageIO
(EnvironmentMap::Load, src/render/EnvironmentMap.cpp:49-92): any readable
image becomes float RGB texels, row 0 at the top, taking channel 0 as red,
channel 1 (else red) as green and channel 2 (else green) as blue; the layout
(lat-long or angular) comes from the caller.  Built without OpenImageIO it
loads nothing.  This module reads the two formats HDR environments ship in:

* Radiance RGBE (``.hdr`` / ``.pic``): ``#?RADIANCE`` / ``#?RGBE`` header,
  ``FORMAT=32-bit_rle_rgbe``, any of the eight resolution-line orientations,
  flat, old-style run-length and new-style (per-component) run-length
  scanlines.  Texels are decoded as ``mantissa * 2^(exponent - 136)`` (the
  rgbe.c convention OpenImageIO's reader uses; exponent 0 is black).
* OpenEXR (``.exr``): single-part scanline images with HALF, FLOAT or UINT
  channels, compression NONE, RLE, ZIPS or ZIP (the zlib-based ones; PIZ,
  PXR24, B44 and DWA are refused with a clear error), any data window and
  line order.  Channels R, G, B are used when present (A is ignored), else a
  luminance channel Y is replicated, else the first channels by name.

``load_environment(path)`` dispatches on the file's magic bytes and returns an
``(height, width, 3)`` float32 array for ``DomeLight.env``.  The importance
tables are then built by the backend at scene upload, as the reference builds
them after loading (EnvironmentMap::BuildImportanceTable, :185-236).
"""
from __future__ import annotations

import re
import struct
import zlib

import numpy as np

__all__ = ["load_environment", "load_hdr", "load_exr", "HdriError"]


class HdriError(ValueError):
    """The file is not a readable HDR environment image."""


# ---------------------------------------------------------------- Radiance --

_RES = re.compile(rb"^([-+])([XY])\s+(\d+)\s+([-+])([XY])\s+(\d+)\s*$")


def _rgbe_to_float(rgbe: np.ndarray) -> np.ndarray:
    """(n, 4) uint8 RGBE -> (n, 3) float32: mantissa * 2^(e - 136), 0 when e == 0."""
    e = rgbe[:, 3].astype(np.int32)
    scale = np.where(e > 0, np.ldexp(np.float32(1.0), e - 136), 0.0).astype(np.float32)
    return rgbe[:, :3].astype(np.float32) * scale[:, None]


def _read_scanline(buf: memoryview, pos: int, width: int) -> tuple:
    """One scanline of RGBE quads starting at buf[pos]; returns (quads, pos)."""
    n = len(buf)
    if 8 <= width <= 0x7FFF and pos + 4 <= n and buf[pos] == 2 and buf[pos + 1] == 2 and not (buf[pos + 2] & 0x80):
        # new-style run-length: four component planes, each of runs / dumps
        if ((buf[pos + 2] << 8) | buf[pos + 3]) != width:
            raise HdriError("RGBE scanline length does not match the image width")
        pos += 4
        line = np.empty((4, width), np.uint8)
        for c in range(4):
            x = 0
            while x < width:
                if pos >= n:
                    raise HdriError("RGBE data ends inside a scanline")
                code = buf[pos]
                pos += 1
                if code > 128:  # run of one value
                    count = code - 128
                    if x + count > width or pos >= n:
                        raise HdriError("RGBE run overflows its scanline")
                    line[c, x:x + count] = buf[pos]
                    pos += 1
                else:  # literal dump
                    count = code
                    if count == 0 or x + count > width or pos + count > n:
                        raise HdriError("RGBE dump overflows its scanline")
                    line[c, x:x + count] = np.frombuffer(buf[pos:pos + count], np.uint8)
                    pos += count
                x += count
        return line.T.copy(), pos
    # flat quads, with old-style runs (1, 1, 1, n) repeating the previous quad
    out = np.empty((width, 4), np.uint8)
    x = 0
    shift = 0
    while x < width:
        if pos + 4 > n:
            raise HdriError("RGBE data ends inside a scanline")
        q = bytes(buf[pos:pos + 4])
        pos += 4
        if q[0] == 1 and q[1] == 1 and q[2] == 1:
            if x == 0:
                raise HdriError("RGBE run at the start of a scanline")
            count = q[3] << shift
            if x + count > width:
                raise HdriError("RGBE run overflows its scanline")
            out[x:x + count] = out[x - 1]
            x += count
            shift += 8
        else:
            out[x] = np.frombuffer(q, np.uint8)
            x += 1
            shift = 0
    return out, pos


def load_hdr(path_or_bytes) -> np.ndarray:
    """A Radiance RGBE image as (height, width, 3) float32, row 0 at the top."""
    data = _read_bytes(path_or_bytes)
    buf = memoryview(data)
    if not (data.startswith(b"#?RADIANCE") or data.startswith(b"#?RGBE") or data.startswith(b"#?")):
        raise HdriError("not a Radiance file (no #? signature)")
    pos = 0
    fmt = None
    while True:  # header: lines up to the first empty one
        end = data.find(b"\n", pos)
        if end < 0:
            raise HdriError("Radiance header is not terminated")
        line = data[pos:end].strip()
        pos = end + 1
        if not line:
            break
        if line.startswith(b"FORMAT="):
            fmt = line[7:].strip()
    if fmt is not None and fmt != b"32-bit_rle_rgbe":
        raise HdriError(f"unsupported Radiance pixel format {fmt.decode(errors='replace')}")
    end = data.find(b"\n", pos)
    if end < 0:
        raise HdriError("Radiance resolution line missing")
    m = _RES.match(data[pos:end].strip())
    if not m or m.group(2) == m.group(5):
        raise HdriError("malformed Radiance resolution line")
    pos = end + 1
    s1, a1, n1, s2, a2, n2 = m.group(1), m.group(2), int(m.group(3)), m.group(4), m.group(5), int(m.group(6))
    if n1 <= 0 or n2 <= 0:
        raise HdriError("empty Radiance image")
    lines = np.empty((n1, n2, 3), np.float32)
    for k in range(n1):
        quads, pos = _read_scanline(buf, pos, n2)
        lines[k] = _rgbe_to_float(quads)
    # map (major, minor) scanlines to rows top-down, columns left-right: the
    # picture's Y axis points up, so "-Y" runs from the top row
    if a1 == b"Y":
        img = lines
        if s1 == b"+":
            img = img[::-1]
        if s2 == b"-":
            img = img[:, ::-1]
    else:
        img = lines.transpose(1, 0, 2)
        if s1 == b"-":
            img = img[:, ::-1]
        if s2 == b"+":
            img = img[::-1]
    return np.ascontiguousarray(img, np.float32)


def _read_bytes(path_or_bytes) -> bytes:
    if isinstance(path_or_bytes, (bytes, bytearray, memoryview)):
        return bytes(path_or_bytes)
    with open(path_or_bytes, "rb") as f:
        return f.read()


# ----------------------------------------------------------------- OpenEXR --

EXR_MAGIC = 20000630
_COMPRESSION = {0: "NONE", 1: "RLE", 2: "ZIPS", 3: "ZIP", 4: "PIZ", 5: "PXR24", 6: "B44", 7: "B44A", 8: "DWAA",
                9: "DWAB"}
_LINES_PER_CHUNK = {0: 1, 1: 1, 2: 1, 3: 16}
_PIXEL_BYTES = {0: 4, 1: 2, 2: 4}  # UINT, HALF, FLOAT
_PIXEL_DTYPE = {0: "<u4", 1: "<f2", 2: "<f4"}


def _exr_header(data: bytes, pos: int) -> tuple:
    """Attributes of a single-part header: {name: (type, raw bytes)}, end."""
    attrs = {}
    while True:
        end = data.find(b"\0", pos)
        if end < 0:
            raise HdriError("OpenEXR header is not terminated")
        name = data[pos:end]
        pos = end + 1
        if not name:
            return attrs, pos
        end = data.find(b"\0", pos)
        if end < 0 or end + 5 > len(data):
            raise HdriError("truncated OpenEXR attribute")
        typ = data[pos:end]
        pos = end + 1
        (size,) = struct.unpack_from("<i", data, pos)
        pos += 4
        if size < 0 or pos + size > len(data):
            raise HdriError("truncated OpenEXR attribute value")
        attrs[name.decode(errors="replace")] = (typ.decode(errors="replace"), data[pos:pos + size])
        pos += size


def _exr_channels(raw: bytes) -> list:
    """chlist: [(name, pixel type, x sampling, y sampling)] in file order."""
    out = []
    pos = 0
    while pos < len(raw):
        end = raw.find(b"\0", pos)
        if end < 0:
            raise HdriError("malformed OpenEXR channel list")
        name = raw[pos:end]
        pos = end + 1
        if not name:
            break
        ptype, _linear, xs, ys = struct.unpack_from("<iB3xii", raw, pos)
        pos += 16
        out.append((name.decode(errors="replace"), ptype, xs, ys))
    return out


def _unpredict_interleave(tmp: np.ndarray) -> bytes:
    """The byte transform shared by ZIP and RLE: undo the delta predictor
    (b[i] = b[i-1] + t[i] - 128) and re-interleave the two halves."""
    if tmp.size == 0:
        return b""
    d = tmp.astype(np.int64)
    d[1:] -= 128
    b = (np.cumsum(d) & 0xFF).astype(np.uint8)
    half = (b.size + 1) // 2
    out = np.empty_like(b)
    out[0::2] = b[:half]
    out[1::2] = b[half:]
    return out.tobytes()


def _rle_decode(packed: bytes, expect: int) -> np.ndarray:
    out = bytearray()
    pos = 0
    n = len(packed)
    while pos < n:
        count = struct.unpack_from("b", packed, pos)[0]
        pos += 1
        if count < 0:
            if pos - count > n:
                raise HdriError("OpenEXR RLE literal overflows its chunk")
            out += packed[pos:pos - count]
            pos -= count
        else:
            if pos >= n:
                raise HdriError("OpenEXR RLE run overflows its chunk")
            out += bytes([packed[pos]]) * (count + 1)
            pos += 1
        if len(out) > expect:
            raise HdriError("OpenEXR RLE chunk decodes past its size")
    return np.frombuffer(bytes(out), np.uint8)


def _decompress(comp: int, packed: bytes, expect: int) -> bytes:
    if len(packed) >= expect:  # stored raw when compression would not shrink it
        return packed[:expect]
    if comp == 0:
        raise HdriError("truncated OpenEXR chunk")
    if comp in (2, 3):
        try:
            tmp = np.frombuffer(zlib.decompress(packed), np.uint8)
        except zlib.error as e:
            raise HdriError(f"OpenEXR zip chunk: {e}") from None
    elif comp == 1:
        tmp = _rle_decode(packed, expect)
    else:
        raise HdriError(f"OpenEXR compression {_COMPRESSION.get(comp, comp)} is not supported")
    if tmp.size != expect:
        raise HdriError("OpenEXR chunk decodes to the wrong size")
    return _unpredict_interleave(tmp)


def _pick_channels(names: list) -> list:
    """Indices of the channels used as R, G, B (OpenImageIO puts R, G, B, A
    first; the reference then replicates missing ones)."""
    def find(want):
        for i, n in enumerate(names):
            if n == want:
                return i
        for i, n in enumerate(names):
            if n.rsplit(".", 1)[-1] == want:
                return i
        return None

    rgb = [find(c) for c in "RGB"]
    if rgb[0] is not None:
        r = rgb[0]
        g = rgb[1] if rgb[1] is not None else r
        b = rgb[2] if rgb[2] is not None else g
        return [r, g, b]
    y = find("Y")
    if y is not None:
        return [y, y, y]
    order = [i for i, n in enumerate(names) if n.rsplit(".", 1)[-1] != "A"] or list(range(len(names)))
    r = order[0]
    g = order[1] if len(order) > 1 else r
    b = order[2] if len(order) > 2 else g
    return [r, g, b]


def load_exr(path_or_bytes) -> np.ndarray:
    """A single-part scanline OpenEXR image (its data window) as (height,
    width, 3) float32, row 0 at the top."""
    data = _read_bytes(path_or_bytes)
    if len(data) < 8:
        raise HdriError("not an OpenEXR file")
    magic, version = struct.unpack_from("<ii", data, 0)
    if magic != EXR_MAGIC:
        raise HdriError("not an OpenEXR file (bad magic number)")
    if (version & 0xFF) != 2:
        raise HdriError(f"unsupported OpenEXR version {version & 0xFF}")
    if version & 0x200:
        raise HdriError("tiled OpenEXR images are not supported")
    if version & (0x800 | 0x1000):
        raise HdriError("deep or multi-part OpenEXR images are not supported")
    attrs, pos = _exr_header(data, 8)
    for need in ("channels", "compression", "dataWindow"):
        if need not in attrs:
            raise HdriError(f"OpenEXR header lacks '{need}'")
    chans = _exr_channels(attrs["channels"][1])
    if not chans:
        raise HdriError("OpenEXR image has no channels")
    for name, ptype, xs, ys in chans:
        if ptype not in _PIXEL_BYTES:
            raise HdriError(f"OpenEXR channel {name}: unknown pixel type {ptype}")
        if xs != 1 or ys != 1:
            raise HdriError(f"OpenEXR channel {name}: subsampled channels are not supported")
    comp = attrs["compression"][1][0]
    if comp not in _LINES_PER_CHUNK:
        raise HdriError(f"OpenEXR compression {_COMPRESSION.get(comp, comp)} is not supported")
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1][:16])
    width, height = x1 - x0 + 1, y1 - y0 + 1
    if width <= 0 or height <= 0:
        raise HdriError("empty OpenEXR data window")
    lpc = _LINES_PER_CHUNK[comp]
    nchunks = (height + lpc - 1) // lpc
    if pos + 8 * nchunks > len(data):
        raise HdriError("truncated OpenEXR offset table")
    offsets = struct.unpack_from(f"<{nchunks}Q", data, pos)
    line_bytes = sum(width * _PIXEL_BYTES[p] for _, p, _, _ in chans)
    planes = [np.zeros((height, width), np.float32) for _ in chans]
    for off in offsets:
        if off + 8 > len(data):
            raise HdriError("OpenEXR chunk offset past the end of the file")
        y, size = struct.unpack_from("<ii", data, off)
        first = y - y0
        if first < 0 or first >= height or first % lpc or size < 0 or off + 8 + size > len(data):
            raise HdriError("malformed OpenEXR chunk")
        lines = min(lpc, height - first)
        raw = _decompress(comp, data[off + 8:off + 8 + size], lines * line_bytes)
        p = 0
        for k in range(lines):
            for c, (_, ptype, _, _) in enumerate(chans):
                nb = width * _PIXEL_BYTES[ptype]
                planes[c][first + k] = np.frombuffer(raw, _PIXEL_DTYPE[ptype], width, p).astype(np.float32)
                p += nb
    idx = _pick_channels([c[0] for c in chans])
    return np.ascontiguousarray(np.stack([planes[i] for i in idx], axis=-1), np.float32)


def load_environment(path_or_bytes) -> np.ndarray:
    """An environment image (Radiance or OpenEXR, told apart by their magic
    bytes) as (height, width, 3) float32 texels for ``DomeLight.env``."""
    data = _read_bytes(path_or_bytes)
    if len(data) >= 4 and struct.unpack_from("<i", data, 0)[0] == EXR_MAGIC:
        return load_exr(data)
    if data.startswith(b"#?"):
        return load_hdr(data)
    raise HdriError("unrecognised image format (expected Radiance .hdr or OpenEXR .exr)")
