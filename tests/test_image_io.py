"""saveImage outputs (materials/Texture.h:44-75): PNG decoded with zlib, EXR parsed from its
scan-line blocks; the pixels must be the reference's conversion of the float image."""
import struct
import zlib

import numpy as np


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, ihdr = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        if typ == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    w, h, depth, color = ihdr[0], ihdr[1], ihdr[2], ihdr[3]
    assert depth == 8 and color == 2
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 3 * w)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 3)


def read_exr(path):
    d = open(path, "rb").read()
    assert struct.unpack("<II", d[:8]) == (20000630, 2)
    pos, attrs = 8, {}
    while d[pos] != 0:
        e = d.index(b"\0", pos)
        name = d[pos:e].decode()
        e2 = d.index(b"\0", e + 1)
        size = struct.unpack("<i", d[e2 + 1:e2 + 5])[0]
        attrs[name] = d[e2 + 5:e2 + 5 + size]
        pos = e2 + 5 + size
    pos += 1
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    assert attrs["compression"] == b"\0"
    offsets = struct.unpack(f"<{h}Q", d[pos:pos + 8 * h])
    img = np.zeros((h, w, 3), np.float32)
    for y, off in enumerate(offsets):
        ly, size = struct.unpack("<ii", d[off:off + 8])
        assert ly == y and size == 12 * w
        line = np.frombuffer(d[off + 8:off + 8 + size], np.float32).reshape(3, w)
        img[y, :, 2], img[y, :, 1], img[y, :, 0] = line  # B, G, R
    return img


def test_png_and_exr(built, tmp_path):
    import narvalengine_gb300 as ne
    rng = np.random.default_rng(0)
    img = rng.uniform(-0.5, 1.5, size=(37, 301, 3)).astype(np.float32)  # > 65535 bytes of scan lines
    img[0, 0] = [np.nan, 1.0, 0.999]
    ne.save_image(str(tmp_path / "a.png"), img)
    ne.save_image(str(tmp_path / "a.exr"), img)
    png = read_png(tmp_path / "a.png")
    want = (np.clip(np.nan_to_num(img, nan=0.0), 0.0, 1.0) * np.float32(255)).astype(np.uint8)
    assert np.array_equal(png, want)
    exr = read_exr(tmp_path / "a.exr")
    assert np.array_equal(exr.view(np.uint32), img.view(np.uint32))
