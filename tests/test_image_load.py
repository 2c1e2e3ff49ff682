"""Texture decoding (ne_image_load_rgba8) against images encoded here with Python's zlib.

The reference loads textures with stbi_load(path, ..., 4) (core/ResourceManager.cpp:288-315):
8-bit RGBA whatever the file holds. Every PNG colour type and bit depth, the five filters,
Adam7 interlacing, palettes with tRNS, colour keys and 16-bit samples are encoded by the small
writer below from known pixels, and the decoded RGBA must equal the rule stb applies.
"""
import os
import struct
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.usefixtures("built")

ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _chunk(t, data):
    return struct.pack(">I", len(data)) + t + data + struct.pack(">I", zlib.crc32(t + data) & 0xFFFFFFFF)


def _pack_line(samples, depth):
    if depth == 8:
        return bytes(int(v) for v in samples)
    if depth == 16:
        return b"".join(struct.pack(">H", int(v)) for v in samples)
    out, acc, nbits = bytearray(), 0, 0
    for v in samples:
        acc = (acc << depth) | int(v)
        nbits += depth
        if nbits == 8:
            out.append(acc)
            acc, nbits = 0, 0
    if nbits:
        out.append(acc << (8 - nbits))
    return bytes(out)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _filter(lines, bpp, first_type):
    out, prev = bytearray(), None
    for k, line in enumerate(lines):
        f = (first_type + k) % 5
        res = bytearray(len(line))
        for i in range(len(line)):
            a = line[i - bpp] if i >= bpp else 0
            b = prev[i] if prev is not None else 0
            c = prev[i - bpp] if (prev is not None and i >= bpp) else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][f]
            res[i] = (line[i] - pred) & 0xFF
        out.append(f)
        out += res
        prev = line
    return bytes(out)


def encode_png(samples, ctype, depth, palette=None, trns=None, interlace=False, level=6, first_filter=0):
    """samples: (H, W, channels) integer array of raw sample values."""
    h, w, ch = samples.shape
    bpp = max(1, (depth * ch + 7) // 8)
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    raw = b""
    for k, (x0, y0, dx, dy) in enumerate(passes):
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        lines = [_pack_line(sub[y].reshape(-1), depth) for y in range(sub.shape[0])]
        raw += _filter(lines, bpp, first_filter + k)
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if palette is not None:
        png += _chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        png += _chunk(b"tRNS", bytes(trns))
    return png + _chunk(b"IDAT", zlib.compress(raw, level)) + _chunk(b"IEND", b"")


def expected_rgba(samples, ctype, depth, palette=None, trns=None):
    s = samples.astype(np.int64)
    h, w, _ = s.shape
    to8 = (lambda v: v >> 8) if depth == 16 else ((lambda v: v) if depth == 8 else (lambda v: v * (255 // ((1 << depth) - 1))))
    out = np.zeros((h, w, 4), np.int64)
    if ctype == 3:
        pal = np.asarray(palette, np.int64)
        out[..., :3] = pal[s[..., 0]]
        alpha = np.full(len(pal), 255, np.int64)
        if trns is not None:
            alpha[:len(trns)] = list(trns)
        out[..., 3] = alpha[s[..., 0]]
        return out.astype(np.uint8)
    if ctype in (0, 4):
        out[..., :3] = to8(s[..., :1])
    else:
        out[..., :3] = to8(s[..., :3])
    out[..., 3] = to8(s[..., -1]) if ctype in (4, 6) else 255
    if trns is not None and ctype in (0, 2):
        key = np.array(struct.unpack(">" + "H" * (len(trns) // 2), bytes(trns)))
        match = np.all(s[..., :len(key)] == key, axis=-1)
        out[..., 3] = np.where(match, 0, out[..., 3])
    return out.astype(np.uint8)


def decode(tmp_path, data, name="t.png"):
    import narvalengine_gb300 as ne
    p = os.path.join(tmp_path, name)
    with open(p, "wb") as f:
        f.write(data)
    return ne.load_image(p)


CASES = [
    # (ctype, depth, interlace, width, height)
    (2, 8, False, 13, 7), (6, 8, False, 9, 11), (0, 8, False, 17, 5), (0, 1, False, 19, 3), (0, 2, False, 11, 6),
    (0, 4, False, 7, 9), (0, 16, False, 5, 5), (4, 8, False, 6, 4), (4, 16, False, 3, 8), (2, 16, False, 10, 3),
    (6, 16, False, 4, 4), (3, 8, False, 12, 5), (3, 4, False, 9, 9), (3, 2, False, 5, 7), (3, 1, False, 33, 2),
    (6, 8, True, 13, 11), (0, 2, True, 10, 9), (3, 4, True, 1, 1), (2, 8, True, 3, 17), (4, 16, True, 9, 2),
]


@pytest.mark.parametrize("ctype,depth,interlace,w,h", CASES)
def test_png_decodes_like_stb(tmp_path, ctype, depth, interlace, w, h):
    rng = np.random.default_rng(ctype * 100 + depth + 7 * interlace)
    ch = CHANNELS[ctype]
    hi = (1 << depth) if ctype != 3 else min(1 << depth, 6)
    samples = rng.integers(0, hi, size=(h, w, ch))
    palette = trns = None
    if ctype == 3:
        palette = rng.integers(0, 256, size=(6, 3))
        trns = [rng.integers(0, 256) for _ in range(3)]  # shorter than the palette: the rest are opaque
    for level, first in ((0, 0), (9, 2)):
        data = encode_png(samples, ctype, depth, palette, trns, interlace, level, first)
        got = decode(tmp_path, data)
        assert got.shape == (h, w, 4)
        assert np.array_equal(got, expected_rgba(samples, ctype, depth, palette, trns)), (ctype, depth, level)


@pytest.mark.parametrize("ctype,depth", [(0, 8), (0, 16), (2, 8), (2, 16)])
def test_png_colour_key(tmp_path, ctype, depth):
    rng = np.random.default_rng(depth)
    ch = CHANNELS[ctype]
    samples = rng.integers(0, 4, size=(6, 8, ch)) * ((1 << depth) // 4)
    key = samples[2, 3]
    trns = b"".join(struct.pack(">H", int(v)) for v in key)
    got = decode(tmp_path, encode_png(samples, ctype, depth, trns=trns))
    want = expected_rgba(samples, ctype, depth, trns=trns)
    assert want[2, 3, 3] == 0
    assert np.array_equal(got, want)


def test_png_large_dynamic_huffman(tmp_path):
    # a smooth 8-bit RGBA gradient with noise compresses into dynamic-Huffman blocks with
    # long back-references
    h, w = 256, 300
    y, x = np.mgrid[0:h, 0:w]
    rng = np.random.default_rng(1)
    img = np.stack([x % 256, y % 256, (x + y) % 256, rng.integers(250, 256, (h, w))], -1)
    got = decode(tmp_path, encode_png(img, 6, 8, level=9))
    assert np.array_equal(got, img.astype(np.uint8))


@pytest.mark.parametrize("magic,maxval", [(b"P6", 255), (b"P5", 255), (b"P6", 1023), (b"P5", 100)])
def test_pnm(tmp_path, magic, maxval):
    rng = np.random.default_rng(maxval)
    ch = 3 if magic == b"P6" else 1
    h, w = 5, 7
    s = rng.integers(0, maxval + 1, size=(h, w, ch))
    body = s.astype(">u2").tobytes() if maxval > 255 else s.astype(np.uint8).tobytes()
    data = magic + b"\n# a comment\n%d %d\n%d\n" % (w, h, maxval) + body
    got = decode(tmp_path, data, "t.ppm")
    v = (s >> 8) if maxval > 255 else s  # samples as stored (high byte of 16-bit ones)
    want = np.concatenate([np.broadcast_to(v, (h, w, 3)) if ch == 1 else v, np.full((h, w, 1), 255)], -1)
    assert np.array_equal(got, want.astype(np.uint8))


def test_load_errors(tmp_path):
    import narvalengine_gb300 as ne
    with pytest.raises(ne.NarvalError) as e:
        ne.load_image(os.path.join(tmp_path, "missing.png"))
    assert e.value.status == -3
    with pytest.raises(ne.NarvalError) as e:
        decode(tmp_path, b"\xff\xd8\xff\xe0" + b"\0" * 64, "t.jpg")
    assert e.value.status == -6
    good = encode_png(np.zeros((4, 4, 3), np.int64), 2, 8)
    with pytest.raises(ne.NarvalError) as e:
        decode(tmp_path, good[:60])
    assert e.value.status == -2


def test_oracle_decoder_agrees_with_the_library(built, tmp_path):
    """The oracle's own texture decoder (oracle/scene_reader.py) against the library's: every
    colour type, bit depth, interlacing, palette with tRNS, colour key and binary PNM decodes to
    the same RGBA8; randomly truncated or altered files are rejected by both or decoded alike."""
    import ctypes as C
    import narvalengine_gb300 as ne
    from oracle.scene_reader import SceneError, _image_rgba8
    lib = ne.library()
    f = tmp_path / "t.img"

    def library(b):
        f.write_bytes(b)
        w, h = C.c_int32(), C.c_int32()
        if lib.ne_image_load_rgba8(str(f).encode(), C.byref(w), C.byref(h), None, 0):
            return None
        out = (C.c_uint8 * (w.value * h.value * 4))()
        if lib.ne_image_load_rgba8(str(f).encode(), C.byref(w), C.byref(h), out, len(out)):
            return None
        return np.frombuffer(out, np.uint8).reshape(h.value, w.value, 4)

    def oracle(b):
        try:
            return _image_rgba8(b)
        except SceneError:
            return None

    rng = np.random.default_rng(12)
    bases = []
    for ct, d, ch in [(0, 1, 1), (0, 2, 1), (0, 4, 1), (0, 8, 1), (0, 16, 1), (2, 8, 3), (2, 16, 3), (3, 1, 1),
                      (3, 2, 1), (3, 4, 1), (3, 8, 1), (4, 8, 2), (4, 16, 2), (6, 8, 4), (6, 16, 4)]:
        for inter in (False, True):
            H, W = int(rng.integers(1, 12)), int(rng.integers(1, 14))
            samp = rng.integers(0, 1 << d, size=(H, W, ch))
            kw = {}
            if ct == 3:
                kw["palette"] = rng.integers(0, 256, size=(int(rng.integers(1, 1 << d)), 3), dtype=np.uint8)
                kw["trns"] = rng.integers(0, 256, size=int(rng.integers(0, 5)), dtype=np.uint8).tobytes()
            elif ct in (0, 2):
                kw["trns"] = b"".join(int(v).to_bytes(2, "big") for v in np.atleast_1d(samp[0, 0]))
            bases.append(encode_png(samp, ct, d, interlace=inter, first_filter=int(rng.integers(0, 5)), **kw))
    bases.append(b"P6\n# comment\n7 5\n255\n" + rng.integers(0, 256, 7 * 5 * 3, dtype=np.uint8).tobytes())
    bases.append(b"P5 4 3 65535 " + rng.integers(0, 256, 4 * 3 * 2, dtype=np.uint8).tobytes())
    for b in bases:
        a, o = library(b), oracle(b)
        assert a is not None and o is not None and np.array_equal(a, o)
    for it in range(600):
        b = bytearray(bases[it % len(bases)])
        if it % 3 == 0:
            b = b[:rng.integers(0, len(b))]
        else:
            for _ in range(rng.integers(1, 4)):
                k = rng.integers(0, len(b))
                b[k] = rng.integers(0, 256) if it % 3 == 1 else b[k] ^ (1 << rng.integers(0, 8))
        a, o = library(bytes(b)), oracle(bytes(b))
        assert (a is None) == (o is None), it
        if a is not None:
            assert np.array_equal(a, o), it
