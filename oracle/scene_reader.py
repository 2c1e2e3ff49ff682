"""The oracle's own reading of the reference's JSON scene descriptor.

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and bench.py's CPU legs,
to build the oracle's scene. The product never imports it.

Restates io/SceneReader.cpp (loadScene :10-54, getVec3 :60-65, processMaterial :67-222,
processPrimitives :224-648, processCameraAndRenderer :650-675), core/Camera.cpp:7-26,
utils/Math.h:848-859 (getTransform, rotate), primitives/InstancedModel.cpp:11-16 (the inverse),
primitives/Triangle.cpp:149-157 (calculateArea), core/ResourceManager.cpp:222-288 (.vol grids)
and :165-218 (.vdb grids, oracle/vdb.py), with glm's arithmetic written out in float32 in glm's own operation order:

* glm::translate, glm::scale and mat4 * mat4 (column j = ((a0 b0j + a1 b1j) + a2 b2j) + a3 b3j);
* glm::eulerAngleXYZ (gtx/euler_angles.inl): the closed form over c_i = cos(-t_i), s_i = sin(-t_i);
* glm::inverse (func_matrix.inl, compute_inverse for 4x4): 18 2x2 minors, the signed cofactor
  columns, one reciprocal of the determinant ((d0 + d1) + (d2 + d3)), scaled;
* glm::normalize(v) = v * (1 / sqrt(dot(v, v))), dot = (x x' + y y') + z z', glm::cross.

It is written from the reference's files and glm's published algorithms, not from the library's
reader (narvalengine_gb300/csrc/scene_host.cpp): the parity tests build the GPU scene with the
library's reader and the oracle's scene with this one, so a mistake in either reading shows up
as a parity failure, and tests/test_oracle_scene_reader.py compares the two descriptions field
by field.

Deviations shared with the library: sin/cos come from the shared elementary functions
(ne_fmath.h, through liboracle.so) and tan(x) is sin(x) / cos(x); the seeded fBm grids and
icospheres of the synthetic configurations come from the seeded generator compiled into
liboracle.so (oracle/inputs.cpp). Descriptor extensions (not in the reference, each opt-in):
"grid" generators and raw ".f32" grids, constant "radiance" environments, "mesh" primitives
(inline or icosphere, optional seeded material "groups"), "obj" read directly, renderer "rr" and
"bvh" — restated from their documented meaning.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import re
import struct
import zlib
from fractions import Fraction

import numpy as np

from narvalengine_gb300 import _abi  # struct layouts only

f32 = np.float32
NE_TEX_ALBEDO, NE_TEX_ROUGHNESS, NE_TEX_METALLIC, NE_TEX_NORMAL, NE_TEX_TEX1 = 1 << 1, 1 << 2, 1 << 3, 1 << 5, 1 << 7
DEFAULT_SEED = 0x4E415256


class SceneError(Exception):
    """A descriptor the reference would reject (LOG(FATAL)) or this reader does not restate."""


def _first_wins(pairs):
    """An object whose repeated keys keep their first value, as rapidjson's FindMember (a
    linear search from the start) finds them."""
    out = {}
    for k, v in pairs:
        out.setdefault(k, v)
    return out


def _no_constant(name):
    """NaN and Infinity are not JSON (a JSON reader rejects them)."""
    raise SceneError(f"bad value {name}")


def _whole(v, lo, hi, what):
    """A whole-number field in [lo, hi], truncated toward zero; else a SceneError."""
    v = float(v)
    if not lo <= v < hi + 1:
        raise SceneError(f"{what} is out of range")
    return int(v)


def _lib():
    from oracle import oracle as orc
    return orc.library()


def _fm(fn: int, x) -> f32:
    """One shared elementary function (ne_fmath.h as compiled into liboracle.so)."""
    a = np.array([x], np.float32)
    o = np.empty(1, np.float32)
    _lib().orc_fmath(fn, C.c_void_p(a.ctypes.data), 1, C.c_void_p(o.ctypes.data))
    return o[0]


def _sin(x):
    return _fm(2, x)


def _cos(x):
    return _fm(3, x)


# ------------------------------------------------------------------ glm in float32
def dot(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def cross(x, y):
    return [x[1] * y[2] - y[1] * x[2], x[2] * y[0] - y[2] * x[0], x[0] * y[1] - y[0] * x[1]]


def normalize(v):
    k = f32(1.0) / np.sqrt(dot(v, v))
    return [v[0] * k, v[1] * k, v[2] * k]


def sub(a, b):
    return [a[0] - b[0], a[1] - b[1], a[2] - b[2]]


def scal(s, v):
    return [s * v[0], s * v[1], s * v[2]]


def neg(v):
    return [-v[0], -v[1], -v[2]]


def identity():
    return [[f32(1.0) if r == c else f32(0.0) for r in range(4)] for c in range(4)]  # m[column][row]


def mat_mul(a, b):
    out = []
    for j in range(4):
        col = []
        for i in range(4):
            s = a[0][i] * b[j][0] + a[1][i] * b[j][1]
            s = s + a[2][i] * b[j][2]
            s = s + a[3][i] * b[j][3]
            col.append(s)
        out.append(col)
    return out


def translate(m, v):
    r = [list(c) for c in m]
    r[3] = [((m[0][i] * v[0] + m[1][i] * v[1]) + m[2][i] * v[2]) + m[3][i] for i in range(4)]
    return r


def scale(m, v):
    return [[m[0][i] * v[0] for i in range(4)], [m[1][i] * v[1] for i in range(4)],
            [m[2][i] * v[2] for i in range(4)], list(m[3])]


def radians(d):
    return f32(d) * f32(0.01745329251994329576923690768489)


def euler_xyz(t1, t2, t3):
    c1, c2, c3 = _cos(-t1), _cos(-t2), _cos(-t3)
    s1, s2, s3 = _sin(-t1), _sin(-t2), _sin(-t3)
    z, one = f32(0.0), f32(1.0)
    return [[c2 * c3, -c1 * s3 + s1 * s2 * c3, s1 * s3 + c1 * s2 * c3, z],
            [c2 * s3, c1 * c3 + s1 * s2 * s3, -s1 * c3 + c1 * s2 * s3, z],
            [-s2, s1 * c2, c1 * c2, z],
            [z, z, z, one]]


def get_transform(t, r, s):
    """utils/Math.h:852-859: translate(I, t) * rotate(r) * scale(s), r in degrees."""
    m = translate(identity(), t)
    m = mat_mul(m, euler_xyz(radians(r[0]), radians(r[1]), radians(r[2])))
    return scale(m, s)


def inverse(m):
    """glm::inverse of a 4x4 (func_matrix.inl compute_inverse), m[column][row]."""
    c00 = m[2][2] * m[3][3] - m[3][2] * m[2][3]
    c02 = m[1][2] * m[3][3] - m[3][2] * m[1][3]
    c03 = m[1][2] * m[2][3] - m[2][2] * m[1][3]
    c04 = m[2][1] * m[3][3] - m[3][1] * m[2][3]
    c06 = m[1][1] * m[3][3] - m[3][1] * m[1][3]
    c07 = m[1][1] * m[2][3] - m[2][1] * m[1][3]
    c08 = m[2][1] * m[3][2] - m[3][1] * m[2][2]
    c10 = m[1][1] * m[3][2] - m[3][1] * m[1][2]
    c11 = m[1][1] * m[2][2] - m[2][1] * m[1][2]
    c12 = m[2][0] * m[3][3] - m[3][0] * m[2][3]
    c14 = m[1][0] * m[3][3] - m[3][0] * m[1][3]
    c15 = m[1][0] * m[2][3] - m[2][0] * m[1][3]
    c16 = m[2][0] * m[3][2] - m[3][0] * m[2][2]
    c18 = m[1][0] * m[3][2] - m[3][0] * m[1][2]
    c19 = m[1][0] * m[2][2] - m[2][0] * m[1][2]
    c20 = m[2][0] * m[3][1] - m[3][0] * m[2][1]
    c22 = m[1][0] * m[3][1] - m[3][0] * m[1][1]
    c23 = m[1][0] * m[2][1] - m[2][0] * m[1][1]
    fac0 = (c00, c00, c02, c03)
    fac1 = (c04, c04, c06, c07)
    fac2 = (c08, c08, c10, c11)
    fac3 = (c12, c12, c14, c15)
    fac4 = (c16, c16, c18, c19)
    fac5 = (c20, c20, c22, c23)
    vec0 = (m[1][0], m[0][0], m[0][0], m[0][0])
    vec1 = (m[1][1], m[0][1], m[0][1], m[0][1])
    vec2 = (m[1][2], m[0][2], m[0][2], m[0][2])
    vec3 = (m[1][3], m[0][3], m[0][3], m[0][3])

    def comb(a, fa, b, fb, c, fc):
        return [(a[k] * fa[k] - b[k] * fb[k]) + c[k] * fc[k] for k in range(4)]

    inv0 = comb(vec1, fac0, vec2, fac1, vec3, fac2)
    inv1 = comb(vec0, fac0, vec2, fac3, vec3, fac4)
    inv2 = comb(vec0, fac1, vec1, fac3, vec3, fac5)
    inv3 = comb(vec0, fac2, vec1, fac4, vec2, fac5)
    sa = (f32(1), f32(-1), f32(1), f32(-1))
    sb = (f32(-1), f32(1), f32(-1), f32(1))
    inv = [[inv0[k] * sa[k] for k in range(4)], [inv1[k] * sb[k] for k in range(4)],
           [inv2[k] * sa[k] for k in range(4)], [inv3[k] * sb[k] for k in range(4)]]
    row0 = (inv[0][0], inv[1][0], inv[2][0], inv[3][0])
    d = [m[0][k] * row0[k] for k in range(4)]
    det = (d[0] + d[1]) + (d[2] + d[3])
    one_over = f32(1.0) / det
    return [[inv[c][r] * one_over for r in range(4)] for c in range(4)]


def flat(m):
    return [m[c][r] for c in range(4) for r in range(4)]


def look_at_camera(position, look_at, vfov, W, H, focus):
    """core/Camera.cpp:7-26 as SceneReader.cpp:650-675 calls it: up (0, 1, 0) and aperture 1e-4
    whatever the file says; tan(x) as sin(x) / cos(x) of the shared elementary functions."""
    position = [f32(x) for x in position]
    look_at = [f32(x) for x in look_at]
    vfov, focus = f32(vfov), f32(focus)
    aspect = f32(W) / f32(H)
    aperture = f32(0.0001)
    up = [f32(0), f32(1), f32(0)]
    half = radians(vfov) / f32(2.0)
    half_h = _sin(half) / _cos(half)
    half_w = aspect * half_h
    front = normalize(sub(position, look_at))
    side = normalize(cross(up, front))
    ll = sub(sub(sub(position, scal(focus * half_w, neg(side))), scal(focus * half_h, up)), scal(focus, neg(front)))
    return dict(position=position, lower_left=ll, horizontal=scal((f32(2.0) * focus) * half_w, neg(side)),
                vertical=scal((f32(2.0) * focus) * half_h, up), side=side, up=up, lens_radius=aperture / f32(2.0))


def camera_struct(position, look_at, vfov, W, H, focus=3.0) -> "_abi.NeCamera":
    """look_at_camera as an ne_camera structure (a view of a batch)."""
    c = look_at_camera(position, look_at, vfov, W, H, focus)
    cam = _abi.NeCamera()
    for key, v in c.items():
        if key == "lens_radius":
            cam.lens_radius = float(v)
        else:
            getattr(cam, key)[:] = [float(x) for x in v]
    return cam


# ------------------------------------------------------------------ JSON helpers
def _need(o: dict, k: str, ctx: str):
    if not isinstance(o, dict) or k not in o:
        raise SceneError(f"{ctx} is missing the property {k}.")
    return o[k]


def get_float(v) -> f32:
    """rapidjson GetFloat(): the double value rounded to float."""
    if isinstance(v, bool):
        return f32(1.0 if v else 0.0)
    if not isinstance(v, (int, float)):
        raise SceneError("not a number")
    return f32(float(v))


def get_vec3(v, default=(0.0, 0.0, 0.0)):
    """SceneReader::getVec3 (:60-65): as many components as the array has (at most three)."""
    if not isinstance(v, list):
        raise SceneError("not an array")
    out = [f32(x) for x in default]
    for i, x in enumerate(v[:3]):
        out[i] = get_float(x)
    return out


_OBJ_DECIMAL = re.compile(r"[+-]?(?:[0-9]+\.?[0-9]*|\.[0-9]+)(?:[eE][+-]?[0-9]+)?")
_OBJ_INTEGER = re.compile(r"[+-]?[0-9]{1,18}")


_STOF = re.compile(r"[ \t\n\v\f\r]*([+-]?)(?:(0[xX](?:[0-9a-fA-F]+\.?[0-9a-fA-F]*|\.[0-9a-fA-F]+)(?:[pP][+-]?[0-9]+)?)"
                   r"|((?:[0-9]+\.?[0-9]*|\.[0-9]+)(?:[eE][+-]?[0-9]+)?)|(inf(?:inity)?|nan))", re.IGNORECASE)


def _nearest_f32(q: Fraction) -> np.float32:
    """The float32 nearest to the rational q (ties to even), as strtof rounds; inf beyond range."""
    if q == 0:
        return np.float32(0.0)
    neg, a = q < 0, abs(q)
    top = np.finfo(np.float32).max
    if a >= Fraction(float(top)) + Fraction(2) ** 103:  # half the last step below 2^128 rounds up
        return np.float32(-np.inf if neg else np.inf)
    with np.errstate(over="ignore"):
        c = np.float32(float(a))  # within one float32 step of the answer
    if np.isinf(c):
        c = top
    cands = [c, np.nextafter(c, np.float32(0))] + ([np.nextafter(c, np.float32(np.inf))] if c < top else [])
    best = None
    for x in cands:
        d = abs(Fraction(float(x)) - a)
        odd = int(np.float32(x).view(np.uint32)) & 1
        key = (d, odd)
        if best is None or key < best[0]:
            best = (key, x)
    x = best[1]
    return np.float32(-x) if neg else np.float32(x)


def _stof_prefix(s: str) -> np.float32:
    """std::stof: leading whitespace skipped, the longest number prefix read (decimal,
    hexadecimal, inf, nan) and rounded to float32 once; no number, or a finite number beyond
    float32's range, is an error (std::stof throws)."""
    m = _STOF.match(s)
    if not m:
        raise SceneError(f"stof: no number in {s[:20]!r}")
    sign = -1 if m.group(1) == "-" else 1
    if m.group(4):
        v = np.float32(float(m.group(1) + m.group(4)))
        return v
    if m.group(3):  # decimal: far outside float32's range, skip the exact arithmetic
        mant, _, exp = m.group(3).lower().partition("e")
        whole, _, frac = mant.partition(".")
        digits = (whole + frac).lstrip("0")
        if not digits:  # a zero, whatever its exponent
            return np.float32(-0.0 if sign < 0 else 0.0)
        if digits:
            lead = len(whole.lstrip("0")) if whole.lstrip("0") else -(len(frac) - len(frac.lstrip("0")))
            mag = int(exp or 0) + lead  # the value is in [10^(mag-1), 10^mag)
            if mag > 40:
                raise SceneError(f"stof: {s[:20]!r} is out of float range")
            if mag < -46:
                return np.float32(-0.0 if sign < 0 else 0.0)
    q = Fraction(float.fromhex(m.group(2))) if m.group(2) else Fraction(m.group(3))
    v = _nearest_f32(sign * q) if q else np.float32(-0.0 if sign < 0 else 0.0)
    if np.isinf(v):
        raise SceneError(f"stof: {s[:20]!r} is out of float range")
    return v


# ------------------------------------------------------------------ image decoding
_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


def _unfilter(raw: bytes, h: int, stride: int, bpp: int) -> np.ndarray:
    """The five PNG scan-line filters undone: h lines of 1 + stride bytes."""
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int64)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int64)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        elif f == 1:  # running sums along each byte lane of a pixel
            cur = np.zeros(stride, np.int64)
            for j in range(min(bpp, stride)):
                cur[j::bpp] = np.cumsum(line[j::bpp]) & 255
        elif f in (3, 4):
            cur = np.zeros(stride, np.int64)
            for i in range(stride):
                a = int(cur[i - bpp]) if i >= bpp else 0
                b = int(prev[i])
                if f == 3:
                    p = (a + b) >> 1
                else:
                    c = int(prev[i - bpp]) if i >= bpp else 0
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[i] = (int(line[i]) + p) & 255
        else:
            raise SceneError("bad PNG filter type")
        out[y] = cur
        prev = cur
    return out


def _samples(lines: np.ndarray, n: int, depth: int) -> np.ndarray:
    """The first n samples of each line (MSB first below 8 bits, big-endian at 16)."""
    if depth == 8:
        return lines[:, :n].astype(np.int64)
    if depth == 16:
        return (lines[:, 0:2 * n:2].astype(np.int64) << 8) | lines[:, 1:2 * n:2]
    bits = np.unpackbits(lines, axis=1)[:, :n * depth].reshape(lines.shape[0], n, depth)
    weights = 1 << np.arange(depth - 1, -1, -1)
    return (bits.astype(np.int64) * weights).sum(2)


def _png_rgba8(data: bytes):
    """PNG to RGBA8 (the texture decoder's rules, as stbi_load(..., 4) gives them): every colour
    type and bit depth, Adam7 interlacing, PLTE/tRNS palettes, tRNS colour keys (on the raw
    samples), grey expanded to RGB, sub-byte grey scaled (x255, x85, x17), 16-bit samples as
    their high byte, a missing alpha 255; chunk CRCs and the zlib checksum are not checked."""
    pos, idat, hdr, plte, trns = 8, b"", None, b"", b""
    while pos + 8 <= len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        if pos + 12 + n > len(data):
            raise SceneError("truncated PNG chunk")
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if typ == b"IHDR" and n >= 13:
            hdr = struct.unpack(">IIBBBBB", body[:13])
        elif typ == b"PLTE":
            plte = body
        elif typ == b"tRNS":
            trns = body
        elif typ == b"IDAT":
            idat += body
        elif typ == b"IEND":
            break
        pos += 12 + n
    if hdr is None or not (1 <= hdr[0] <= 65536 and 1 <= hdr[1] <= 65536):
        raise SceneError("bad PNG header")
    w, h, depth, ctype, _, _, interlace = hdr
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}.get(ctype)
    if chans is None:
        raise SceneError("bad PNG colour type")
    ok = (ctype != 3 or depth == 8) if depth in (8, 16) else (depth in (1, 2, 4) and ctype in (0, 3))
    if not ok or interlace > 1 or (ctype == 3 and not plte):
        raise SceneError("unsupported PNG bit depth, palette or interlace method")
    if len(idat) < 2 or (idat[0] & 0x0F) != 8 or ((idat[0] << 8) | idat[1]) % 31 or (idat[1] & 0x20):
        raise SceneError("bad zlib header")
    dec = zlib.decompressobj(-15)
    try:
        raw = dec.decompress(idat[2:])
    except zlib.error as e:
        raise SceneError(f"corrupt deflate stream: {e}")
    if not dec.eof:
        raise SceneError("truncated deflate stream")
    to8 = (lambda v: v >> 8) if depth == 16 else (lambda v: v) if depth == 8 else \
        (lambda v: v * (255 // ((1 << depth) - 1)))
    key = lambda k: (trns[2 * k] << 8) | trns[2 * k + 1]
    out = np.zeros((h, w, 4), np.uint8)
    off = 0
    for x0, y0, dx, dy in (_ADAM7 if interlace else ((0, 0, 1, 1),)):
        pw = (w - x0 + dx - 1) // dx if w > x0 else 0
        ph = (h - y0 + dy - 1) // dy if h > y0 else 0
        if pw == 0 or ph == 0:
            continue
        stride = (pw * depth * chans + 7) // 8
        if off + ph * (stride + 1) > len(raw):
            raise SceneError("PNG image data too short")
        lines = _unfilter(raw[off:off + ph * (stride + 1)], ph, stride, max(1, depth * chans // 8))
        off += ph * (stride + 1)
        s = _samples(lines, pw * chans, depth).reshape(ph, pw, chans)
        px = np.zeros((ph, pw, 4), np.int64)
        if ctype in (0, 4):
            px[..., 0] = px[..., 1] = px[..., 2] = to8(s[..., 0])
            px[..., 3] = to8(s[..., 1]) if ctype == 4 else 255
            if ctype == 0 and len(trns) >= 2:
                px[..., 3][s[..., 0] == key(0)] = 0
        elif ctype == 2:
            px[..., :3] = to8(s)
            px[..., 3] = 255
            if len(trns) >= 6:
                px[..., 3][(s[..., 0] == key(0)) & (s[..., 1] == key(1)) & (s[..., 2] == key(2))] = 0
        elif ctype == 3:
            k = s[..., 0]
            pal = np.zeros((256, 3), np.int64)
            m = len(plte) // 3
            pal[:m] = np.frombuffer(plte[:3 * m], np.uint8).reshape(m, 3)
            alpha = np.full(256, 255, np.int64)
            alpha[:len(trns)] = np.frombuffer(trns[:256], np.uint8)
            px[..., :3] = np.where((3 * k + 2 < len(plte))[..., None], pal[np.minimum(k, 255)], 0)
            px[..., 3] = alpha[np.minimum(k, 255)]
        else:
            px[...] = to8(s)
        out[y0::dy, x0::dx][:ph, :pw] = px.astype(np.uint8)
    return out


def _pnm_rgba8(data: bytes):
    """Binary PNM (P5 grey, P6 RGB): width, height and maxval after whitespace and '#' comments,
    one byte, then the samples as stored (16-bit samples by their first, high, byte)."""
    pos = 2
    vals = []
    for _ in range(3):
        while True:
            while pos < len(data) and data[pos] in b" \t\n\r":
                pos += 1
            if pos < len(data) and data[pos] == ord("#"):
                while pos < len(data) and data[pos] != ord("\n"):
                    pos += 1
                continue
            break
        if pos >= len(data) or not 48 <= data[pos] <= 57:
            raise SceneError("bad PNM header")
        v = 0
        while pos < len(data) and 48 <= data[pos] <= 57:
            v = v * 10 + data[pos] - 48
            pos += 1
            if v > 0xFFFFFFFF:
                raise SceneError("bad PNM header")
        vals.append(v)
    w, h, maxval = vals
    if not (1 <= w <= 65536 and 1 <= h <= 65536 and 1 <= maxval <= 65535):
        raise SceneError("bad PNM header")
    pos += 1
    ch = 3 if data[1:2] == b"6" else 1
    nb = 2 if maxval > 255 else 1
    need = w * h * ch * nb
    if pos + need > len(data):
        raise SceneError("PNM data too short")
    s = np.frombuffer(data, np.uint8, need, pos).reshape(h * w, ch, nb)[:, :, 0]
    out = np.full((h * w, 4), 255, np.uint8)
    out[:, :3] = s if ch == 3 else s[:, :1]
    return out.reshape(h, w, 4)


def _image_rgba8(data: bytes):
    """A texture file as RGBA8: PNG by its signature, binary PNM by "P5" / "P6"."""
    if data[:8] == b"\x89PNG\r\n\x1a\n":
        return _png_rgba8(data)
    if len(data) >= 3 and data[:1] == b"P" and data[1:2] in (b"5", b"6"):
        return _pnm_rgba8(data)
    raise SceneError("only PNG and binary PNM (P5/P6) images are decoded")


# ------------------------------------------------------------------ the reader
class OracleSceneDesc:
    """A scene read by the oracle: `desc` (ne_scene_desc) and the arrays it points into."""

    def __init__(self, path: str | None = None, text: str | None = None, resources_dir: str | None = None):
        if text is None:
            if not os.path.exists(path):
                raise SceneError(f"Couldn't read {path}.")
            text = open(path).read()
            if resources_dir is None:
                resources_dir = os.path.dirname(os.path.abspath(path))
        self.res_dir = resources_dir or ""
        self.instances, self.light_instances = [], []
        self.models, self.prims, self.materials, self.model_materials = [], [], [], []
        self.lights, self.media, self.grids, self.textures = [], [], [], []
        self.mat_by_name = {}
        self.obj_models = {}
        self.mesh_arrays = []
        self.n_prims = 0  # primitives so far (a mesh entry of `prims` holds many)
        try:
            doc = json.loads(text, parse_constant=_no_constant, object_pairs_hook=_first_wins)
        except (ValueError, RecursionError) as e:
            raise SceneError(f"malformed json: {e}")
        self._load(doc)
        self._finalize()

    # io/SceneReader.cpp:10-54
    def _load(self, doc):
        if not isinstance(doc, dict):
            raise SceneError("Malformatted json file. Not a valid json object.")
        if "version" not in doc:
            raise SceneError("Incomplete json file. Version is not present.")
        for m in _need(doc, "materials", "scene"):
            self._material(m)
        for p in _need(doc, "primitives", "scene"):
            self._primitive(p)
        self._camera_renderer(_need(doc, "camera", "scene"), _need(doc, "renderer", "scene"))

    def _asset(self, rel: str) -> str:
        if rel.startswith("/") or not self.res_dir:
            return rel
        return os.path.join(self.res_dir, rel)

    def _new_light(self, **kw):
        L = dict(type=0, primitive=-1, li=[f32(0)] * 3, le=[f32(0)] * 3, direction=[f32(0)] * 3,
                 env_radiance=[f32(0)] * 3, env_map_pdf=f32(0), env=None)
        L.update(kw)
        self.lights.append(L)
        return len(self.lights) - 1

    # io/SceneReader.cpp:67-222 processMaterial
    def _material(self, m):
        name = _need(m, "name", "Material")
        typ = _need(m, "type", f"Material {name}")
        ctx = f"Material {name}"
        mat = dict(bsdf=0, light=-1, medium=-1, phase=0, g=f32(0), albedo=[f32(0)] * 3, roughness=f32(0),
                   metallic=f32(0), normal_map=[f32(0)] * 3, tex_present=0, tex_types=0, albedo_tex=None)
        if typ == "microfacet":
            alb = _need(m, "albedo", ctx)
            if isinstance(alb, str):
                # :80-103: the texture loaded by ResourceManager::loadTexture as RGBA8; the constant
                # keeps its default (1, 0, 1)
                mat["albedo"] = [f32(1), f32(0), f32(1)]
                w, h, rgba = self._load_rgba8(alb, ctx)
                self.textures.append(np.ascontiguousarray(rgba))
                mat["albedo_tex"] = (w, h, len(self.textures) - 1)
            else:
                mat["albedo"] = get_vec3(alb, (1.0, 0.0, 1.0))
            has_normal = "normalMap" in m
            mat["normal_map"] = get_vec3(m["normalMap"], (0, 0, 1)) if has_normal else [f32(0), f32(0), f32(1)]
            mat["roughness"] = get_float(_need(m, "roughness", ctx))
            mat["metallic"] = get_float(_need(m, "metallic", ctx))
            mat["bsdf"] = 1
            # Material::addTexture (materials/Material.h:38-44) for ALBEDO, METALLIC, ROUGHNESS[,
            # NORMAL]: every slot is set, textureTypes = the last type added
            mat["tex_present"] = NE_TEX_ALBEDO | NE_TEX_METALLIC | NE_TEX_ROUGHNESS | (NE_TEX_NORMAL if has_normal else 0)
            mat["tex_types"] = NE_TEX_NORMAL if has_normal else NE_TEX_ROUGHNESS
        elif typ == "emitter":
            li = get_vec3(_need(m, "albedo", ctx))
            mat["light"] = self._new_light(type=0, li=li)
            mat["albedo"] = list(li)
            mat["tex_present"] = mat["tex_types"] = NE_TEX_ALBEDO
        elif typ == "directionalLight":
            le = get_vec3(_need(m, "albedo", ctx))
            pos = get_vec3(_need(m, "position", ctx))
            direction = normalize(sub([f32(0)] * 3, pos))
            mat["light"] = self._new_light(type=1, le=le, direction=direction)
        elif typ == "infiniteAreaLight":
            if "path" in m:
                w, h, rgba = self._load_rgba8(m["path"], ctx)
                if h > w:
                    raise SceneError(f"{ctx}: environment maps taller than wide read past the image in the reference")
                self.textures.append(np.ascontiguousarray(rgba))
                mat["light"] = self._new_light(type=2, env=(w, h, len(self.textures) - 1))
            else:
                rad = get_vec3(_need(m, "radiance", ctx))
                # a 1x1 map of that value: Distribution2D gives pdf func/funcInt = 1 when the green
                # channel is positive, else 0 (lights/InfiniteAreaLight.h:20-40, utils/Sampling.h:12-28)
                mat["light"] = self._new_light(type=2, env_radiance=rad,
                                               env_map_pdf=f32(1.0) if rad[1] > 0 else f32(0.0))
            mat["tex_present"] = mat["tex_types"] = NE_TEX_TEX1
        elif typ == "volume":
            md = dict(type=1, sigma_s=get_vec3(_need(m, "scattering", ctx)),
                      sigma_a=get_vec3(_need(m, "absorption", ctx)), density=f32(0), res=[0, 0, 0], grid=None)
            pf = _need(m, "phaseFunction", ctx)
            if pf == "isotropic":
                mat["phase"] = 0
            elif pf in ("hg", "henyey-greenstein"):
                mat["phase"] = 1
                mat["g"] = get_float(_need(m, "g", ctx))
            else:
                raise SceneError(f"{ctx}: unknown phase function {pf}")
            md["density"] = get_float(_need(m, "density", ctx))
            with np.errstate(over="ignore", invalid="ignore"):
                for a in range(3):
                    ss, sa = md["sigma_s"][a], md["sigma_a"][a]
                    if not (np.isfinite((ss + sa) * md["density"]) and np.isfinite(ss) and np.isfinite(sa)):
                        raise SceneError(f"{ctx}: scattering, absorption and density must stay finite")
            if "path" in m:
                path = m["path"]
                if ".vdb" in path:  # core/ResourceManager.cpp:165-218 loadVDBasTexture
                    from oracle.vdb import VdbError, load_density
                    try:
                        md["res"], md["grid"] = load_density(self._asset(path))
                    except VdbError as e:
                        raise SceneError(f"{ctx}: {e}")
                elif ".vol" in path:
                    md["res"], md["grid"] = self._load_vol(path)
                else:
                    raise SceneError(f"{ctx}: volume path must be a .vol or .vdb file")
                md["type"] = 0
            elif "grid" in m:
                md["res"], md["grid"] = self._grid_extension(m["grid"], ctx)
                md["type"] = 0
            self.media.append(md)
            mat["medium"] = len(self.media) - 1
            mat["bsdf"] = 2
            mat["tex_present"] = mat["tex_types"] = NE_TEX_TEX1
        else:
            raise SceneError("Invalid material type while reading scene from json file.")
        self.materials.append(mat)
        self.mat_by_name[name] = len(self.materials) - 1

    def _load_rgba8(self, rel, ctx):
        full = self._asset(rel)
        if not os.path.exists(full):
            raise SceneError(f"{ctx}: missing texture {rel}")
        img = _image_rgba8(open(full, "rb").read())
        return img.shape[1], img.shape[0], img

    def _load_vol(self, path):
        """core/ResourceManager.cpp:222-288: line 1 "X Y Z " (each value ended by a space), line 2
        skipped, then the remaining lines joined with "\\n" and cut at spaces; each piece is read by
        std::stof (a piece that spans a line break gives its first number only)."""
        full = self._asset(path)
        if not os.path.exists(full):
            raise SceneError(f"Couldn't read the file at {full}.")
        lines = open(full, "rb").read().decode("latin-1").split("\n")
        first = lines[0]
        pieces = first.split(" ")[:-1]
        if len(pieces) < 3:
            raise SceneError(f"volume {path}: resolution line needs three values")
        res = [_whole(np.float32(_stof_prefix(x)), 1, 65536, f"volume {path} resolution") for x in pieces[:3]]
        total = res[0] * res[1] * res[2]
        grid = np.zeros(total, np.float32)
        data = "".join(ln + "\n" for ln in lines[2:])
        vals = data.split(" ")[:-1]
        if len(vals) > total:
            raise SceneError(f"volume {path}: more values than the resolution")
        for k, v in enumerate(vals):
            grid[k] = np.float32(_stof_prefix(v))
        return res, grid

    def _grid_extension(self, g, ctx):
        res_f = get_vec3(_need(g, "resolution", ctx + " grid"))
        if not all(1.0 <= float(x) < 65537.0 for x in res_f):
            raise SceneError(f"{ctx}: grid resolution must be 1 to 65536 voxels per axis")
        res = [int(x) for x in res_f]
        n = res[0] * res[1] * res[2]
        if "path" in g:
            full = self._asset(g["path"])
            if not os.path.exists(full):
                raise SceneError(f"Couldn't read the file at {full}.")
            grid = np.fromfile(full, dtype="<f4", count=n)
            if grid.size != n:
                raise SceneError(f"grid {g['path']}: file shorter than the resolution")
            return res, grid.astype(np.float32)
        if g.get("generator") != "fbm":
            raise SceneError(f"{ctx}: unknown grid generator")
        octaves, seed = float(g.get("octaves", 5)), float(g.get("seed", DEFAULT_SEED))
        if not 1.0 <= octaves < 33.0:
            raise SceneError(f"{ctx}: grid octaves must be 1 to 32")
        if not 0.0 <= seed <= 2.0 ** 53:
            raise SceneError(f"{ctx}: grid seed must be an integer from 0 to 2^53")
        grid = np.empty(n, np.float32)
        r3 = (C.c_uint32 * 3)(*res)
        _lib().orc_gen_fbm(r3, int(g.get("octaves", 5)), float(g.get("frequency", 4.0 / res[0])),
                           float(g.get("lacunarity", 2.0)), float(g.get("gain", 0.5)),
                           float(g.get("falloff_radius", res[0] * 0.5)), int(g.get("seed", DEFAULT_SEED)),
                           C.c_void_p(grid.ctypes.data))
        return res, grid

    def _material_named(self, name, ctx):
        if name not in self.mat_by_name:
            raise SceneError(f"{ctx}: unknown material {name}")
        return self.mat_by_name[name]

    def _add_instance(self, M, model, collision, is_light):
        inst = dict(to_wcs=flat(M), to_ocs=flat(inverse(M)), model=model, collision=1 if collision else 0)
        (self.light_instances if is_light else self.instances).append(inst)

    def _single_prim_model(self, prim, mat, emissive):
        """A Model of one primitive in Model::lights (emissive material) or Model::primitives,
        with Model::materials = [material]; the light's primitive is that primitive."""
        prim["material"] = mat
        self.prims.append(prim)
        pi = self.n_prims
        self.n_prims += 1
        md = dict(prim_begin=pi, prim_count=0 if emissive else 1, light_begin=pi, light_count=1 if emissive else 0,
                  mat_begin=len(self.model_materials), mat_count=1, has_bbox=0, bbox_min=[f32(0)] * 3,
                  bbox_max=[f32(0)] * 3, use_bvh=0)
        if emissive:
            self.lights[self.materials[mat]["light"]]["primitive"] = pi
        self.model_materials.append(mat)
        self.models.append(md)
        return len(self.models) - 1

    @staticmethod
    def _prim(typ, p0=(0, 0, 0), p1=(0, 0, 0), p2=(0, 0, 0), radius=0.0, area=0.0):
        return dict(type=typ, material=-1, p0=[f32(x) for x in p0], p1=[f32(x) for x in p1],
                    p2=[f32(x) for x in p2], radius=f32(radius), area=f32(area))

    # io/SceneReader.cpp:224-648 processPrimitives
    def _primitive(self, p):
        name = _need(p, "name", "Primitive")
        ctx = f"Primitive {name}"
        typ = _need(p, "type", ctx)
        tr = _need(p, "transform", ctx)
        pos = get_vec3(_need(tr, "position", ctx + " transform"))
        collision = bool(p.get("collision", True))

        def sr():
            return (get_vec3(_need(tr, "scale", ctx + " transform"), (1, 1, 1)),
                    get_vec3(_need(tr, "rotation", ctx + " transform")))

        if typ == "point":  # :267-325
            s, r = sr()
            mat = self._material_named(_need(p, "materialName", ctx), ctx)
            em = self.materials[mat]["light"] >= 0
            mi = self._single_prim_model(self._prim(4, p0=pos), mat, em)
            self._add_instance(get_transform(pos, r, s), mi, True, em)
        elif typ == "sphere":  # :326-380: centre at the OCS origin, translation only
            radius = get_float(_need(p, "radius", ctx))
            mat = self._material_named(_need(p, "materialName", ctx), ctx)
            em = self.materials[mat]["light"] >= 0
            mi = self._single_prim_model(self._prim(0, radius=radius), mat, em)
            self._add_instance(get_transform(pos, [f32(0)] * 3, [f32(1)] * 3), mi, collision, em)
        elif typ == "rectangle":  # :381-494: vertexData[0] = point1, vertexData[1] = vertex 2, normal (0,0,-1)
            s, r = sr()
            mat = self._material_named(_need(p, "materialName", ctx), ctx)
            em = self.materials[mat]["light"] >= 0
            prim = self._prim(1, p0=(-0.5, -0.5, 0.0), p1=(0.5, 0.5, 0.0), p2=(0.0, 0.0, -1.0))
            mi = self._single_prim_model(prim, mat, em)
            self._add_instance(get_transform(pos, r, s), mi, True, em)
        elif typ == "volume":  # :495-642: AABB from point1f (-0.5) to point1b (0.5)
            s, r = sr()
            mat = self._material_named(_need(p, "materialName", ctx), ctx)
            mi = self._single_prim_model(self._prim(2, p0=(-0.5,) * 3, p1=(0.5,) * 3), mat, False)
            self._add_instance(get_transform(pos, r, s), mi, True, False)
        elif typ == "mesh":  # extension
            s, r = sr()
            self._mesh(p, ctx)
            self._add_instance(get_transform(pos, r, s), len(self.models) - 1, collision, False)
        elif typ == "obj":  # :245-266; the InstancedModel keeps isCollisionEnabled = true
            s, r = sr()
            path = _need(p, "path", ctx)
            if "materialName" not in p:
                raise SceneError(f"{ctx}: obj models need a materialName")
            key = (path, p["materialName"])
            if key not in self.obj_models:
                vpos, vidx = self._read_obj(self._asset(path), ctx)
                self._mesh_model(vpos, vidx, p, ctx)
                self.obj_models[key] = len(self.models) - 1
            self._add_instance(get_transform(pos, r, s), self.obj_models[key], True, False)
        elif typ == "gltf":
            raise SceneError(f"{ctx}: gltf models are not restated")
        else:
            raise SceneError("Invalid primitive type while reading scene from json file.")

    def _mesh(self, p, ctx):
        if "generator" in p:
            if p["generator"] != "icosphere":
                raise SceneError(f"{ctx}: unknown mesh generator")
            if not 0.0 <= float(p.get("subdivisions", 3)) < 11.0:
                raise SceneError(f"{ctx}: subdivisions must be 0 to 10")
            n = int(p.get("subdivisions", 3))
            d = p.get("displacement", {})
            amp, freq = float(d.get("amplitude", 0.0)), float(d.get("frequency", 1.0))
            if not 0.0 <= float(d.get("seed", DEFAULT_SEED)) <= 2.0 ** 53:
                raise SceneError(f"{ctx}: displacement seed must be an integer from 0 to 2^53")
            seed = int(d.get("seed", DEFAULT_SEED))
            nv, nt = 10 * 4 ** n + 2, 20 * 4 ** n
            pos = np.empty(nv * 3, np.float32)
            idx = np.empty(nt * 3, np.uint32)
            _lib().orc_gen_icosphere(n, amp, freq, seed, C.c_void_p(pos.ctypes.data), C.c_void_p(idx.ctypes.data))
        else:
            pos = np.array([float(x) for x in _need(p, "positions", ctx)], np.float32)
            idx = np.array([int(x) for x in _need(p, "indices", ctx)], np.int64)
            if pos.size % 3 or idx.size % 3:
                raise SceneError(f"{ctx}: positions/indices not multiples of 3")
            if idx.size and (idx.min() < 0 or idx.max() * 3 + 2 >= pos.size):
                raise SceneError(f"{ctx}: index out of range")
            idx = idx.astype(np.uint32)
        self._mesh_model(pos, idx, p, ctx)

    def _read_obj(self, path, ctx):
        """Wavefront positions and faces ("v x y z"; "f a b c ..." with a, a/t, a/t/n or a//n,
        1-based or negative); polygons become fans (v0, vi, vi+1), as assimp triangulates convex
        faces. Lines split at "\\n" (one trailing "\\r" dropped), tokens at spaces and tabs; a first
        token starting with "#" is a comment, other keywords are ignored; a vertex needs three
        decimal numbers (read as double, then float32), a face three vertex indices (a signed
        integer before any "/")."""
        if not os.path.exists(path):
            raise SceneError(f"{ctx}: cannot open {path}")
        pos, idx = [], []
        for n, ln in enumerate(open(path, "rb").read().decode("latin-1").split("\n"), 1):
            if ln.endswith("\r"):
                ln = ln[:-1]
            t = [x for x in re.split(r"[ \t]", ln) if x]
            if not t or t[0].startswith("#"):
                continue
            if t[0] == "v":
                if len(t) < 4 or not all(_OBJ_DECIMAL.fullmatch(x) for x in t[1:4]):
                    raise SceneError(f"{ctx}: bad vertex at line {n}")
                pos.extend(np.float32(float(x)) for x in t[1:4])
            elif t[0] == "f":
                nv = len(pos) // 3
                face = []
                for tok in t[1:]:
                    head = tok.split("/")[0]
                    if not _OBJ_INTEGER.fullmatch(head):
                        raise SceneError(f"{ctx}: bad face at line {n}")
                    v = int(head)
                    vi = v - 1 if v > 0 else nv + v
                    if vi < 0 or vi >= nv:
                        raise SceneError(f"{ctx}: face index out of range at line {n}")
                    face.append(vi)
                if len(face) < 3:
                    raise SceneError(f"{ctx}: face with fewer than 3 vertices at line {n}")
                for k in range(1, len(face) - 1):
                    idx += [face[0], face[k], face[k + 1]]
        return np.array(pos, np.float32), np.array(idx, np.uint32)

    def _mesh_model(self, pos, idx, p, ctx):
        """A triangle Model (primitives/Model.cpp:4-7, 337-370): one primitive per triangle,
        bounding box over the triangles' vertices, a BVH; material from "materialName" or the
        seeded "groups" extension (group k: roughness and albedo uniform in the given ranges from
        the seeded hash, draws 4k and 4k+1; triangle t in group t * count / n)."""
        nt = idx.size // 3
        if nt == 0:
            raise SceneError(f"{ctx}: mesh has no triangles")
        md = dict(prim_begin=self.n_prims, prim_count=nt, light_begin=self.n_prims + nt, light_count=0,
                  mat_begin=len(self.model_materials), mat_count=0, has_bbox=1, use_bvh=1)
        if "groups" in p:
            gr = p["groups"]
            count = _whole(get_float(gr.get("count", 1)), 1, 65536, f"{ctx} group count")
            rr = [f32(x) for x in gr.get("roughness", [0.05, 0.9])]
            ar = [f32(x) for x in gr.get("albedo", [0.2, 0.9])]
            seed = _whole(gr.get("seed", DEFAULT_SEED), 0, 2 ** 53, f"{ctx} group seed")
            first = len(self.materials)
            for k in range(count):
                u0 = _lib().orc_gen_hash_u01(seed, 4 * k)
                u1 = _lib().orc_gen_hash_u01(seed, 4 * k + 1)
                rough = f32(float(rr[0]) + float(rr[1] - rr[0]) * u0)
                a = f32(float(ar[0]) + float(ar[1] - ar[0]) * u1)
                self.materials.append(dict(bsdf=1, light=-1, medium=-1, phase=0, g=f32(0), albedo=[a, a, a],
                                           roughness=rough, metallic=f32(0), normal_map=[f32(0)] * 3,
                                           tex_present=NE_TEX_ALBEDO | NE_TEX_METALLIC | NE_TEX_ROUGHNESS,
                                           tex_types=NE_TEX_ROUGHNESS))
                self.model_materials.append(first + k)
            tri_mat = first + (np.arange(nt, dtype=np.uint64) * np.uint64(count) // np.uint64(nt)).astype(np.int64)
            md["mat_count"] = count
        elif "materialName" in p:
            mat = self._material_named(p["materialName"], ctx)
            tri_mat = np.full(nt, mat, np.int64)
            self.model_materials.append(mat)
            md["mat_count"] = 1
        else:
            tri_mat = np.full(nt, -1, np.int64)
        v = pos.reshape(-1, 3)[idx.reshape(-1, 3)]  # (nt, 3 vertices, 3)
        a, b, c = v[:, 0], v[:, 1], v[:, 2]
        e1, e2 = b - a, c - a
        n = np.stack([e1[:, 1] * e2[:, 2] - e2[:, 1] * e1[:, 2], e1[:, 2] * e2[:, 0] - e2[:, 2] * e1[:, 0],
                      e1[:, 0] * e2[:, 1] - e2[:, 0] * e1[:, 1]], 1)
        area = np.sqrt((n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]) / np.float32(2.0)
        seq = v.reshape(-1, 3)
        mn, mx = [], []
        for c_ in range(3):
            col = seq[:, c_]
            lo, hi = col.min(), col.max()
            mn.append(col[np.argmax(col == lo)])  # first occurrence keeps the sign of a zero
            mx.append(col[np.argmax(col == hi)])
        md["bbox_min"], md["bbox_max"] = mn, mx
        self.mesh_arrays.append((v.astype(np.float32), tri_mat, area.astype(np.float32)))
        # the mesh's triangles are one entry of `prims` (expanded in _finalize)
        self.prims.append(("mesh", len(self.mesh_arrays) - 1))
        self.n_prims += nt
        self.models.append(md)

    # io/SceneReader.cpp:650-675 and core/Camera.cpp:7-26
    def _camera_renderer(self, cam, ren):
        position = get_vec3(_need(cam, "position", "camera"))
        look_at = get_vec3(_need(cam, "lookAt", "camera"))
        vfov = get_float(_need(cam, "vfov", "camera"))
        res = _need(ren, "resolution", "renderer")
        if not isinstance(res, list) or len(res) < 2:
            raise SceneError("renderer resolution needs [W, H]")
        if not (float(res[0]) >= 1.0 and float(res[1]) >= 1.0):
            raise SceneError("renderer resolution must be positive")
        W, H = _whole(res[0], 1, 2 ** 31 - 1, "renderer resolution"), _whole(res[1], 1, 2 ** 31 - 1, "renderer resolution")
        if cam.get("autoFocus") is True:
            focus = f32(3.0)  # (position - lookAt).length() is glm's component count
        else:
            focus = get_float(_need(cam, "focus", "camera"))
        self.camera = look_at_camera(position, look_at, vfov, W, H, focus)
        st = dict(width=W, height=H, spp=_whole(get_float(_need(ren, "spp", "renderer")), -2 ** 31, 2 ** 31 - 1, "spp"),
                  bounces=_whole(get_float(_need(ren, "bounces", "renderer")), -2 ** 31, 2 ** 31 - 1, "bounces"),
                  hdr=1 if ren.get("HDR") is True else 0,
                  rr_enabled=0, rr_after=3, bvh_build=0)
        if "rr" in ren:
            st["rr_enabled"] = 1
            if "after" in ren["rr"]:
                st["rr_after"] = _whole(get_float(ren["rr"]["after"]), -2 ** 31, 2 ** 31 - 1, "rr after")
        if "bvh" in ren:
            if ren["bvh"] == "sah":
                st["bvh_build"] = 1
            elif ren["bvh"] != "reference":
                raise SceneError('renderer bvh must be "reference" or "sah"')
        self.settings = st

    # ---------------------------------------------------------------- ctypes description
    def _finalize(self):
        A = _abi
        insts = self.instances + self.light_instances
        self._inst = (A.NeInstance * max(1, len(insts)))()
        for i, x in enumerate(insts):
            self._inst[i].to_wcs[:] = [float(v) for v in x["to_wcs"]]
            self._inst[i].to_ocs[:] = [float(v) for v in x["to_ocs"]]
            self._inst[i].model = x["model"]
            self._inst[i].collision = x["collision"]
        self._models = (A.NeModel * max(1, len(self.models)))()
        for i, md in enumerate(self.models):
            for k in ("prim_begin", "prim_count", "light_begin", "light_count", "mat_begin", "mat_count",
                      "has_bbox", "use_bvh"):
                setattr(self._models[i], k, md[k])
            self._models[i].bbox_min[:] = [float(v) for v in md["bbox_min"]]
            self._models[i].bbox_max[:] = [float(v) for v in md["bbox_max"]]
        # primitives: single ones and mesh blocks, in order
        n_prims = self.n_prims
        prim_dtype = np.dtype([("type", "<i4"), ("material", "<i4"), ("p", "<f4", (3, 3)), ("radius", "<f4"),
                               ("area", "<f4")])
        assert prim_dtype.itemsize == C.sizeof(A.NePrimitive)
        parr = np.zeros(max(1, n_prims), prim_dtype)
        k = 0
        for e in self.prims:
            if isinstance(e, tuple):
                v, tri_mat, area = self.mesh_arrays[e[1]]
                n = v.shape[0]
                parr["type"][k:k + n] = 3
                parr["material"][k:k + n] = tri_mat
                parr["p"][k:k + n] = v
                parr["area"][k:k + n] = area
                k += n
            else:
                parr[k]["type"] = e["type"]
                parr[k]["material"] = e["material"]
                parr[k]["p"] = np.array([e["p0"], e["p1"], e["p2"]], np.float32)
                parr[k]["radius"] = e["radius"]
                parr[k]["area"] = e["area"]
                k += 1
        self._prims_np = parr
        self._mats = (A.NeMaterial * max(1, len(self.materials)))()
        for i, m in enumerate(self.materials):
            o = self._mats[i]
            for key in ("bsdf", "light", "medium", "phase", "tex_present", "tex_types"):
                setattr(o, key, m[key])
            o.g, o.roughness, o.metallic = float(m["g"]), float(m["roughness"]), float(m["metallic"])
            o.albedo[:] = [float(v) for v in m["albedo"]]
            o.normal_map[:] = [float(v) for v in m["normal_map"]]
            if m.get("albedo_tex") is not None:
                w, h, ti = m["albedo_tex"]
                o.albedo_width, o.albedo_height = w, h
                o.albedo_texels = self.textures[ti].ctypes.data_as(C.POINTER(C.c_uint8))
        self._mm = (C.c_uint32 * max(1, len(self.model_materials)))(*self.model_materials)
        self._lights = (A.NeLight * max(1, len(self.lights)))()
        for i, L in enumerate(self.lights):
            o = self._lights[i]
            o.type, o.primitive = L["type"], L["primitive"]
            for key in ("li", "le", "direction", "env_radiance"):
                getattr(o, key)[:] = [float(v) for v in L[key]]
            o.env_map_pdf = float(L["env_map_pdf"])
            if L["env"] is not None:
                w, h, ti = L["env"]
                o.env_width, o.env_height = w, h
                o.env_texels = self.textures[ti].ctypes.data_as(C.POINTER(C.c_uint8))
        self._media = (A.NeMedium * max(1, len(self.media)))()
        for i, md in enumerate(self.media):
            o = self._media[i]
            o.type = md["type"]
            o.sigma_s[:] = [float(v) for v in md["sigma_s"]]
            o.sigma_a[:] = [float(v) for v in md["sigma_a"]]
            o.density = float(md["density"])
            o.res[:] = md["res"]
            if md["grid"] is not None:
                self.grids.append(md["grid"])
                o.grid = md["grid"].ctypes.data_as(C.POINTER(C.c_float))
        d = A.NeSceneDesc()
        d.n_instances, d.n_light_instances = len(self.instances), len(self.light_instances)
        d.instances = self._inst
        d.n_models, d.models = len(self.models), self._models
        d.n_prims = n_prims
        d.prims = C.cast(C.c_void_p(parr.ctypes.data), C.POINTER(A.NePrimitive))
        d.n_materials, d.materials = len(self.materials), self._mats
        d.n_model_materials, d.model_materials = len(self.model_materials), self._mm
        d.n_lights, d.lights = len(self.lights), self._lights
        d.n_media, d.media = len(self.media), self._media
        for key, v in self.camera.items():
            if key == "lens_radius":
                d.camera.lens_radius = float(v)
            else:
                getattr(d.camera, key)[:] = [float(x) for x in v]
        for key, v in self.settings.items():
            setattr(d.settings, key, v)
        self.desc = d

    @property
    def desc_ptr(self):
        return C.pointer(self.desc)

    @property
    def width(self):
        return self.desc.settings.width

    @property
    def height(self):
        return self.desc.settings.height

    @property
    def spp(self):
        return self.desc.settings.spp

    @property
    def bounces(self):
        return self.desc.settings.bounces
