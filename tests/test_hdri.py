"""Environment images from disk without OpenImageIO (shiro_gb300/hdri.py).

The files are written here byte by byte after the published formats
(Radiance RGBE with flat, old-style and new-style run-length scanlines;
OpenEXR scanline files with NONE, RLE, ZIPS and ZIP chunks, whose zlib / RLE
stages follow OpenEXR's byte reordering and delta predictor) and read back;
values whose encoding is exact must come back bit for bit, RGBE within its
8-bit mantissa.
"""
import struct
import zlib

import numpy as np
import pytest

from shiro_gb300 import hdri

# ------------------------------------------------------------------ RGBE ----


def float_to_rgbe(img):
    """rgbe.c float2rgbe: v = max component; (v < 1e-32) -> 0; mantissa
    scale 256 / 2^e with frexp's exponent, stored exponent e + 128."""
    flat = img.reshape(-1, 3).astype(np.float64)
    v = flat.max(axis=1)
    m, e = np.frexp(v)
    out = np.zeros((flat.shape[0], 4), np.uint8)
    ok = v >= 1e-32
    scale = np.where(ok, m * 256.0 / np.where(ok, v, 1.0), 0.0)
    out[:, :3] = np.where(ok[:, None], np.floor(flat * scale[:, None]), 0).astype(np.uint8)
    out[:, 3] = np.where(ok, e + 128, 0).astype(np.uint8)
    return out.reshape(img.shape[0], img.shape[1], 4)


def rgbe_decode_ref(q):
    """What a texel must read as: mantissa * 2^(e - 136)."""
    out = np.zeros(q.shape[:-1] + (3,), np.float32)
    e = q[..., 3].astype(np.int32)
    for c in range(3):
        out[..., c] = np.where(e > 0, q[..., c].astype(np.float64) * np.ldexp(1.0, e - 136), 0.0)
    return out


def new_rle_line(q):
    """One scanline in new-style run-length form (runs of >= 3 as runs)."""
    w = q.shape[0]
    out = bytearray([2, 2, w >> 8, w & 0xFF])
    for c in range(4):
        comp = q[:, c]
        x = 0
        while x < w:
            run = 1
            while x + run < w and run < 127 and comp[x + run] == comp[x]:
                run += 1
            if run >= 3:
                out += bytes([128 + run, comp[x]])
                x += run
                continue
            start = x
            while x < w and x - start < 128:
                if x + 2 < w and comp[x] == comp[x + 1] == comp[x + 2]:
                    break
                x += 1
            out += bytes([x - start]) + comp[start:x].tobytes()
    return bytes(out)


def old_rle_line(q):
    """Flat quads with old-style repeat records (1, 1, 1, n)."""
    out = bytearray()
    x = 0
    while x < q.shape[0]:
        out += q[x].tobytes()
        run = 0
        while x + 1 + run < q.shape[0] and run < 255 and (q[x + 1 + run] == q[x]).all():
            run += 1
        if run:
            out += bytes([1, 1, 1, run])
        x += 1 + run
    return bytes(out)


def hdr_bytes(q, style="new", res=None, header=b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0\n\n"):
    h, w = q.shape[:2]
    out = bytearray(header)
    out += res if res is not None else f"-Y {h} +X {w}\n".encode()
    for y in range(h):
        line = q[y]
        out += {"new": new_rle_line, "old": old_rle_line, "flat": lambda l: l.tobytes()}[style](line)
    return bytes(out)


@pytest.fixture(scope="module")
def texels():
    rng = np.random.default_rng(5)
    img = np.exp(rng.normal(0.0, 2.0, (13, 40, 3))).astype(np.float32)
    img[0, :10] = 0.0          # black run
    img[3, 5:30] = img[3, 5]   # long run
    img[7, 7] = 1e4            # sun
    return float_to_rgbe(img)


@pytest.mark.parametrize("style", ["new", "old", "flat"])
def test_hdr_scanline_styles(texels, style):
    got = hdri.load_hdr(hdr_bytes(texels, style))
    np.testing.assert_array_equal(got, rgbe_decode_ref(texels))


def test_hdr_orientations(texels):
    want = rgbe_decode_ref(texels)
    h, w = texels.shape[:2]
    # "+Y" stores the bottom row first; "-X" stores columns right to left
    flipped = texels[::-1]
    got = hdri.load_hdr(hdr_bytes(flipped, "flat", res=f"+Y {h} +X {w}\n".encode()))
    np.testing.assert_array_equal(got, want)
    mirrored = texels[:, ::-1]
    got = hdri.load_hdr(hdr_bytes(mirrored, "flat", res=f"-Y {h} -X {w}\n".encode()))
    np.testing.assert_array_equal(got, want)
    # column-major: "+X w -Y h" stores column 0 first, top to bottom
    cols = np.ascontiguousarray(texels.transpose(1, 0, 2))
    got = hdri.load_hdr(hdr_bytes(cols, "flat", res=f"+X {w} -Y {h}\n".encode()))
    np.testing.assert_array_equal(got, want)


def test_hdr_known_texels():
    # (128, 64, 32, 129): 128 * 2^-7 = 1, 0.5, 0.25; exponent 0 -> black
    q = np.array([[[128, 64, 32, 129], [255, 0, 1, 0], [1, 2, 3, 136]]], np.uint8)
    got = hdri.load_hdr(hdr_bytes(q, "flat"))
    np.testing.assert_array_equal(got[0], np.array([[1.0, 0.5, 0.25], [0, 0, 0], [1, 2, 3]], np.float32))
    assert hdri.load_environment(hdr_bytes(q, "flat")).shape == (1, 3, 3)


def test_hdr_errors(texels):
    with pytest.raises(hdri.HdriError):
        hdri.load_hdr(b"#?RADIANCE\nFORMAT=32-bit_rle_xyze\n\n-Y 1 +X 1\n\0\0\0\0")
    with pytest.raises(hdri.HdriError):
        hdri.load_hdr(hdr_bytes(texels, "new")[:-10])  # truncated
    with pytest.raises(hdri.HdriError):
        hdri.load_hdr(b"#?RADIANCE\n\n-Y 2 -Y 2\n")
    with pytest.raises(hdri.HdriError):
        hdri.load_environment(b"P6\n1 1\n255\n\0\0\0")


# ---------------------------------------------------------------- OpenEXR ----

HALF, FLOAT, UINT = 1, 2, 0
DTYPE = {HALF: "<f2", FLOAT: "<f4", UINT: "<u4"}
LINES = {0: 1, 1: 1, 2: 1, 3: 16}


def attr(name, typ, value):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(value)) + value


def predict_reorder(raw):
    """OpenEXR's zip / rle preprocessing: even bytes to the first half, odd to
    the second, then each byte stored as its difference to the previous + 128."""
    b = np.frombuffer(raw, np.uint8)
    t = np.concatenate([b[0::2], b[1::2]]).astype(np.int64)
    d = t.copy()
    d[1:] = (t[1:] - t[:-1] + 128 + 256) & 0xFF
    return d.astype(np.uint8).tobytes()


def rle_encode(data):
    out = bytearray()
    i = 0
    n = len(data)
    while i < n:
        run = 1
        while i + run < n and run < 128 and data[i + run] == data[i]:
            run += 1
        if run >= 3:
            out += struct.pack("b", run - 1) + data[i:i + 1]
            i += run
            continue
        start = i
        while i < n and i - start < 127:
            if i + 2 < n and data[i] == data[i + 1] == data[i + 2]:
                break
            i += 1
        out += struct.pack("b", -(i - start)) + data[start:i]
    return bytes(out)


def exr_bytes(planes, comp=0, window=(0, 0), decreasing=False, force_raw=False):
    """planes: {name: (2-D array, pixel type)}; channels stored by name."""
    names = sorted(planes)
    h, w = next(iter(planes.values()))[0].shape
    x0, y0 = window
    ch = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", planes[n][1], 0, 1, 1) for n in names) + b"\0"
    head = struct.pack("<ii", 20000630, 2)
    head += attr("channels", "chlist", ch)
    head += attr("compression", "compression", bytes([comp]))
    head += attr("dataWindow", "box2i", struct.pack("<iiii", x0, y0, x0 + w - 1, y0 + h - 1))
    head += attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1))
    head += attr("lineOrder", "lineOrder", bytes([1 if decreasing else 0]))
    head += attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
    head += attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
    head += attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
    head += b"\0"
    lpc = LINES[comp]
    chunks = []
    for first in range(0, h, lpc):
        raw = b"".join(np.ascontiguousarray(planes[n][0][y], DTYPE[planes[n][1]]).tobytes()
                       for y in range(first, min(h, first + lpc)) for n in names)
        if comp in (2, 3):
            packed = zlib.compress(predict_reorder(raw))
        elif comp == 1:
            packed = rle_encode(predict_reorder(raw))
        else:
            packed = raw
        if force_raw or len(packed) >= len(raw):
            packed = raw
        chunks.append(struct.pack("<ii", y0 + first, len(packed)) + packed)
    order = list(range(len(chunks)))
    if decreasing:
        order = order[::-1]
    table_end = len(head) + 8 * len(chunks)
    offsets = [0] * len(chunks)
    body = b""
    for k in order:
        offsets[k] = table_end + len(body)
        body += chunks[k]
    return head + struct.pack(f"<{len(chunks)}Q", *offsets) + body


@pytest.fixture(scope="module")
def rgb():
    rng = np.random.default_rng(3)
    img = np.exp(rng.normal(0.0, 1.5, (37, 29, 3))).astype(np.float32)
    img[5:9, :] = 0.25   # flat rows compress well
    img[10, 3] = 3.0e4
    return img


@pytest.mark.parametrize("comp", [0, 1, 2, 3])
@pytest.mark.parametrize("ptype", [HALF, FLOAT])
def test_exr_compressions_and_types(rgb, comp, ptype):
    want = rgb.astype(np.float16).astype(np.float32) if ptype == HALF else rgb
    planes = {c: (want[..., i], ptype) for i, c in enumerate("RGB")}
    planes["A"] = (np.ones(want.shape[:2], np.float32), ptype)
    got = hdri.load_exr(exr_bytes(planes, comp))
    np.testing.assert_array_equal(got, want)
    assert hdri.load_environment(exr_bytes(planes, comp)).shape == want.shape


def test_exr_window_order_raw_chunks_and_uint(rgb):
    planes = {c: (rgb[..., i], FLOAT) for i, c in enumerate("RGB")}
    for kw in (dict(window=(-4, 7)), dict(decreasing=True), dict(comp=3, force_raw=True), dict(comp=1, decreasing=True)):
        np.testing.assert_array_equal(hdri.load_exr(exr_bytes(planes, **kw)), rgb)
    counts = np.arange(12, dtype=np.uint32).reshape(3, 4) * 1000
    got = hdri.load_exr(exr_bytes({"R": (counts, UINT), "G": (counts, UINT), "B": (counts, UINT)}, 2))
    np.testing.assert_array_equal(got[..., 0], counts.astype(np.float32))


def test_exr_channel_choice(rgb):
    y = rgb[..., 1]
    got = hdri.load_exr(exr_bytes({"Y": (y, FLOAT)}))
    np.testing.assert_array_equal(got, np.stack([y, y, y], -1))
    got = hdri.load_exr(exr_bytes({"R": (rgb[..., 0], FLOAT)}))  # R only: G and B repeat it
    np.testing.assert_array_equal(got, np.stack([rgb[..., 0]] * 3, -1))
    got = hdri.load_exr(exr_bytes({"diffuse.R": (rgb[..., 0], FLOAT), "diffuse.G": (rgb[..., 1], FLOAT),
                                   "diffuse.B": (rgb[..., 2], FLOAT)}))
    np.testing.assert_array_equal(got, rgb)


def test_exr_known_bytes():
    """A 2x1 FLOAT image written out field by field: R = (1, 2), G = (3, 4), B = (5, 6)."""
    planes = {"R": (np.array([[1.0, 2.0]], np.float32), FLOAT), "G": (np.array([[3.0, 4.0]], np.float32), FLOAT),
              "B": (np.array([[5.0, 6.0]], np.float32), FLOAT)}
    data = exr_bytes(planes, 0)
    # chunk: y = 0, 24 bytes: B line, G line, R line (channels in name order)
    tail = struct.pack("<ii", 0, 24) + struct.pack("<6f", 5, 6, 3, 4, 1, 2)
    assert data.endswith(tail)
    np.testing.assert_array_equal(hdri.load_exr(data)[0], [[1, 3, 5], [2, 4, 6]])


def test_exr_refusals(rgb):
    planes = {c: (rgb[..., i], HALF) for i, c in enumerate("RGB")}
    data = bytearray(exr_bytes(planes, 0))
    piz = bytearray(data)
    i = piz.find(b"compression\0compression\0")
    piz[i + 28] = 4  # PIZ
    with pytest.raises(hdri.HdriError, match="PIZ"):
        hdri.load_exr(bytes(piz))
    tiled = bytearray(data)
    tiled[4:8] = struct.pack("<i", 2 | 0x200)
    with pytest.raises(hdri.HdriError, match="tiled"):
        hdri.load_exr(bytes(tiled))
    with pytest.raises(hdri.HdriError):
        hdri.load_exr(bytes(data[:-40]))
    with pytest.raises(hdri.HdriError):
        hdri.load_exr(b"\x76\x2f\x31\x01\x02\0\0\0")


def test_loaded_environment_renders_on_the_cpu_checker(rgb):
    """A loaded image is an ordinary dome texture: the environment tables of
    the oracle accept it."""
    import oracle
    from oracle import api

    env = hdri.load_exr(exr_bytes({c: (rgb[..., i], HALF) for i, c in enumerate("RGB")}, 3))
    row, cond = api.env_tables(oracle.port_checker(), env)
    assert row[-1] == pytest.approx(1.0) and np.all(np.diff(row) >= 0)


def test_hdr_header_variants(texels):
    # "#?RGBE" signature, comment and extra variable lines, no FORMAT line
    data = hdr_bytes(texels, "new", header=b"#?RGBE\n# made by a test\nGAMMA=1.0\nSOFTWARE=x\n\n")
    np.testing.assert_array_equal(hdri.load_hdr(data), rgbe_decode_ref(texels))


def test_exr_random_line_order_and_extra_attributes(rgb):
    planes = {c: (rgb[..., i], HALF) for i, c in enumerate("RGB")}
    data = bytearray(exr_bytes(planes, 3))
    # a reader must not depend on attribute order or unknown attributes: insert
    # one before the end of the header, shifting the offsets accordingly
    extra = attr("owner", "string", b"test")
    end = data.index(b"screenWindowWidth\0float\0") + len(b"screenWindowWidth\0float\0") + 4 + 4
    assert data[end] == 0
    nchunks = (rgb.shape[0] + 15) // 16
    offs = list(struct.unpack_from(f"<{nchunks}Q", data, end + 1))
    shifted = bytes(data[:end]) + extra + b"\0" + struct.pack(f"<{nchunks}Q", *[o + len(extra) for o in offs]) + \
        bytes(data[end + 1 + 8 * nchunks:])
    want = rgb.astype(np.float16).astype(np.float32)
    np.testing.assert_array_equal(hdri.load_exr(shifted), want)
    # lineOrder RANDOM_Y: chunks located through the offset table only
    rnd = bytearray(shifted)
    i = rnd.index(b"lineOrder\0lineOrder\0") + len(b"lineOrder\0lineOrder\0") + 4
    rnd[i] = 2
    np.testing.assert_array_equal(hdri.load_exr(bytes(rnd)), want)


# ------------------------------------------- the native (C ABI) reader -------

def _native(data):
    """shiro_hdri_decode of libshiro_gpu.so (host code, no device)."""
    import ctypes as C

    from shiro_gb300 import build
    from shiro_gb300.backend import load_library

    build.build()
    lib = load_library()
    lib.shiro_hdri_decode.argtypes = [C.c_char_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p,
                                      C.c_size_t]
    lib.shiro_hdri_decode.restype = C.c_int
    lib.shiro_hdri_free.argtypes = [C.c_void_p]
    w, h = C.c_uint32(), C.c_uint32()
    px = C.POINTER(C.c_float)()
    err = C.create_string_buffer(256)
    rc = lib.shiro_hdri_decode(bytes(data), len(data), C.byref(w), C.byref(h), C.byref(px), err, 256)
    if rc != 0:
        return None, err.value.decode()
    img = np.ctypeslib.as_array(px, shape=(h.value * w.value * 3,)).copy().reshape(h.value, w.value, 3)
    lib.shiro_hdri_free(C.cast(px, C.c_void_p))
    return img, ""


def _native_cases(texels, rgb):
    h, w = texels.shape[:2]
    yield "hdr new", hdr_bytes(texels, "new")
    yield "hdr old", hdr_bytes(texels, "old")
    yield "hdr flat", hdr_bytes(texels, "flat")
    yield "hdr +Y", hdr_bytes(texels[::-1], "flat", res=f"+Y {h} +X {w}\n".encode())
    yield "hdr -X", hdr_bytes(texels[:, ::-1], "flat", res=f"-Y {h} -X {w}\n".encode())
    yield "hdr cols", hdr_bytes(np.ascontiguousarray(texels.transpose(1, 0, 2)), "flat", res=f"+X {w} -Y {h}\n".encode())
    yield "hdr cols rev", hdr_bytes(np.ascontiguousarray(texels.transpose(1, 0, 2)[::-1, ::-1]), "flat",
                                    res=f"-X {w} +Y {h}\n".encode())
    yield "hdr header", hdr_bytes(texels, "new", header=b"#?RGBE\n# comment\nGAMMA=1.0\n\n")
    for comp in (0, 1, 2, 3):
        for ptype in (HALF, FLOAT):
            want = rgb.astype(np.float16).astype(np.float32) if ptype == HALF else rgb
            planes = {c: (want[..., i], ptype) for i, c in enumerate("RGB")}
            planes["A"] = (np.ones(want.shape[:2], np.float32), ptype)
            yield f"exr comp {comp} type {ptype}", exr_bytes(planes, comp)
    planes = {c: (rgb[..., i], FLOAT) for i, c in enumerate("RGB")}
    for k, kw in enumerate((dict(window=(-4, 7)), dict(decreasing=True), dict(comp=3, force_raw=True),
                            dict(comp=1, decreasing=True))):
        yield f"exr layout {k}", exr_bytes(planes, **kw)
    counts = np.arange(12, dtype=np.uint32).reshape(3, 4) * 1000 + 7
    yield "exr uint", exr_bytes({"R": (counts, UINT), "G": (counts, UINT), "B": (counts, UINT)}, 2)
    yield "exr Y", exr_bytes({"Y": (rgb[..., 1], FLOAT)}, 3)
    yield "exr R only", exr_bytes({"R": (rgb[..., 0], FLOAT)}, 1)
    yield "exr layers", exr_bytes({"diffuse.R": (rgb[..., 0], FLOAT), "diffuse.G": (rgb[..., 1], FLOAT),
                                   "diffuse.B": (rgb[..., 2], FLOAT)}, 2)
    specials = np.array([[0.0, -0.0, 6.1e-5, 5.96e-8, 65504.0, np.inf, -2.5, 1.0]], np.float16).astype(np.float32)
    yield "exr half specials", exr_bytes({c: (specials, HALF) for c in "RGB"}, 0)
    big = np.exp(np.random.default_rng(9).normal(0.0, 1.0, (80, 300, 3))).astype(np.float32)
    yield "exr zip big", exr_bytes({c: (big[..., i], HALF) for i, c in enumerate("RGB")}, 3)


def test_native_reader_equals_the_python_reader(texels, rgb):
    """The C ABI's reader (for C++ hosts: EnvironmentMap::Load's counterpart)
    returns exactly what shiro_gb300.hdri returns, file for file."""
    for name, data in _native_cases(texels, rgb):
        want = hdri.load_environment(data)
        got, err = _native(data)
        assert got is not None, (name, err)
        assert got.shape == want.shape, name
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), name


def test_native_reader_refuses_what_the_python_reader_refuses(rgb):
    planes = {c: (rgb[..., i], HALF) for i, c in enumerate("RGB")}
    data = bytearray(exr_bytes(planes, 0))
    piz = bytearray(data)
    i = piz.find(b"compression\0compression\0")
    piz[i + 28] = 4
    tiled = bytearray(data)
    tiled[4:8] = struct.pack("<i", 2 | 0x200)
    zipd = bytearray(exr_bytes(planes, 3))
    for bad, word in ((bytes(piz), "compression"), (bytes(tiled), "tiled"), (bytes(data[:-40]), ""),
                      (b"\x76\x2f\x31\x01\x02\0\0\0", ""), (b"P6\n1 1\n255\n\0\0\0", "unrecognised"),
                      (b"#?RADIANCE\nFORMAT=32-bit_rle_xyze\n\n-Y 1 +X 1\n\0\0\0\0", "format"),
                      (bytes(zipd[:-5]), "")):
        got, err = _native(bad)
        assert got is None and word in err, (word, err)
        with pytest.raises(hdri.HdriError):
            hdri.load_environment(bad)
