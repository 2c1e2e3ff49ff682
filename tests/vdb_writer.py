"""OpenVDB files for the tests (no OpenVDB here): a writer of OpenVDB 6.2's file layout for float
grids (as io/Archive.cc writeHeader / writeGrid, GridDescriptor writeHeader / writeStreamPos,
the nodes' writeTopology / writeBuffers and io/Compression.h writeCompressedValues lay them out),
with zip, raw and Blosc-1 chunks (stored, or LZ4 streams from a small greedy encoder, byte
shuffled, in one stream per block or one per byte of the type, in one block or several), and the
dense array loadVDBasTexture (core/ResourceManager.cpp:165-218) makes of such a grid, computed
from the sparse description by painting its parts into a numpy box.

A grid is described sparsely: a background, root tiles {origin (multiple of 4096): (value,
active)}, 128^3 tiles {origin (multiple of 128): (value, active)}, 8^3 tiles {origin (multiple of
8): (value, active)} and leaves {origin (multiple of 8): (512 values, 512 active flags)} in the
leaf's x-major order (x * 64 + y * 8 + z). Internal nodes are made where tiles or leaves below
them need them; their other entries are inactive background tiles.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

MAGIC = 0x56444220


class Grid:
    def __init__(self, background=0.0, name="density", half=False):
        self.name = name
        self.background = np.float32(background)
        self.half = half
        self.root_tiles = {}
        self.tiles128 = {}
        self.tiles8 = {}
        self.leaves = {}

    def leaf(self, origin, values, active):
        self.leaves[tuple(origin)] = (np.asarray(values, np.float32).reshape(512),
                                      np.asarray(active, bool).reshape(512))

    # ------------------------------------------------------------------ expected result
    def stored(self, v):
        """A value as the file holds it (half floats for a _HalfFloat grid)."""
        v = np.asarray(v, np.float32)
        return v.astype(np.float16).astype(np.float32) if self.half else v

    def active_box(self):
        lo, hi = np.full(3, np.iinfo(np.int64).max), np.full(3, np.iinfo(np.int64).min)
        any_ = False
        for table, size in ((self.root_tiles, 4096), (self.tiles128, 128), (self.tiles8, 8)):
            for o, (_, a) in table.items():
                if a:
                    lo, hi, any_ = np.minimum(lo, o), np.maximum(hi, np.add(o, size - 1)), True
        for o, (_, act) in self.leaves.items():
            idx = np.nonzero(act)[0]
            if idx.size:
                pts = np.stack([idx >> 6, (idx >> 3) & 7, idx & 7], 1) + np.asarray(o)
                lo, hi, any_ = np.minimum(lo, pts.min(0)), np.maximum(hi, pts.max(0)), True
        return (lo, hi) if any_ else None

    def expected(self):
        """(res, grid) of loadVDBasTexture: the box from -|min| with |min| + |max| voxels per axis
        (one more across 0), z fastest; res = (dim z, dim y, dim x)."""
        lo, hi = self.active_box()
        dim = [int(abs(lo[a]) + abs(hi[a]) + (1 if lo[a] < 0 <= hi[a] else 0)) for a in range(3)]
        org = [-int(abs(lo[a])) for a in range(3)]
        box = np.full(dim, self.background, np.float32)

        def paint(o, size, value):
            a = [max(o[k], org[k]) - org[k] for k in range(3)]
            b = [min(o[k] + size, org[k] + dim[k]) - org[k] for k in range(3)]
            if all(a[k] < b[k] for k in range(3)):
                box[a[0]:b[0], a[1]:b[1], a[2]:b[2]] = value

        for o, (v, _) in self.root_tiles.items():
            paint(o, 4096, np.float32(v))
        for o in self._nodes5():  # a node's unlisted entries are background tiles
            paint(o, 4096, self.background)
        for o, (v, _) in self.tiles128.items():
            paint(o, 128, self.stored(v))
        for o in self._nodes4():
            paint(o, 128, self.background)
        for o, (v, _) in self.tiles8.items():
            paint(o, 8, self.stored(v))
        for o, (vals, act) in self.leaves.items():
            # every value as stored (inactive values and backgrounds in the tests are exact in half)
            block = self.stored(vals).reshape(8, 8, 8)
            a = [max(o[k], org[k]) for k in range(3)]
            b = [min(o[k] + 8, org[k] + dim[k]) for k in range(3)]
            if all(a[k] < b[k] for k in range(3)):
                box[a[0] - org[0]:b[0] - org[0], a[1] - org[1]:b[1] - org[1], a[2] - org[2]:b[2] - org[2]] = \
                    block[a[0] - o[0]:b[0] - o[0], a[1] - o[1]:b[1] - o[1], a[2] - o[2]:b[2] - o[2]]
        return [dim[2], dim[1], dim[0]], box.reshape(-1)

    # ------------------------------------------------------------------ tree
    def _nodes4(self):
        keys = set(self.tiles8) | set(self.leaves)
        return sorted({tuple(c & ~127 for c in o) for o in keys})

    def _nodes5(self):
        keys = set(self.tiles128) | set(self._nodes4())
        return sorted({tuple(c & ~4095 for c in o) for o in keys})


# ---------------------------------------------------------------------- compression
def lz4_encode(data: bytes) -> bytes:
    """A valid LZ4 block: greedy matches of at least 4 bytes found through a hash of 4 bytes."""
    out = bytearray()
    n, i, anchor = len(data), 0, 0
    table = {}

    def length(v):
        while v >= 255:
            out.append(255)
            v -= 255
        out.append(v)

    while i + 4 <= n:
        key = data[i:i + 4]
        j = table.get(key)
        table[key] = i
        if j is not None and i - j <= 65535:
            m = 4
            while i + m < n and data[j + m] == data[i + m]:
                m += 1
            lit = i - anchor
            out.append((min(lit, 15) << 4) | min(m - 4, 15))
            if lit >= 15:
                length(lit - 15)
            out += data[anchor:i]
            out += struct.pack("<H", i - j)
            if m - 4 >= 15:
                length(m - 4 - 15)
            i += m
            anchor = i
        else:
            i += 1
    lit = n - anchor
    out.append(min(lit, 15) << 4)
    if lit >= 15:
        length(lit - 15)
    out += data[anchor:]
    return bytes(out)


def blosc_frame(data: bytes, mode: str, typesize: int = 4) -> bytes:
    """mode: "stored" (flag 2), "lz4" (byte shuffle, one stream per block), "lz4split" (byte
    shuffle, one stream per byte of the type), "raw" (one stream stored raw inside the frame),
    "blocks" (LZ4 in 256-byte blocks, the last one shorter)."""
    n = len(data)
    if mode == "stored":
        body = data
        flags = 0x02 | 0x01
        return bytes([2, 1, flags, typesize]) + struct.pack("<III", n, n, 16 + n) + body
    blocksize = min(256, n) if mode == "blocks" else n  # Blosc never makes a block larger than the data
    nblocks = -(-n // blocksize) if n else 0
    flags = (1 << 5) | 0x01 | (0 if mode == "lz4split" else 0x10)
    blocks = []
    for j in range(nblocks):
        chunk = data[j * blocksize:(j + 1) * blocksize]
        count = len(chunk) // typesize
        body = np.frombuffer(chunk[:count * typesize], np.uint8).reshape(count, typesize).T.tobytes() + \
            chunk[count * typesize:]
        last = j == nblocks - 1 and n % blocksize != 0
        nsplit = typesize if (mode == "lz4split" and len(chunk) // typesize >= 128 and not last) else 1
        neblock = len(body) // nsplit
        streams = b""
        for s in range(nsplit):
            part = body[s * neblock:(s + 1) * neblock]
            enc = part if mode == "raw" else lz4_encode(part)
            if len(enc) == neblock and mode != "raw":
                enc = part  # an incompressible stream is stored raw
            streams += struct.pack("<i", len(enc)) + enc
        blocks.append(streams)
    at = 16 + 4 * nblocks
    starts = []
    for b in blocks:
        starts.append(at)
        at += len(b)
    body = struct.pack(f"<{nblocks}i", *starts) + b"".join(blocks)
    return bytes([2, 1, flags, typesize]) + struct.pack("<III", n, blocksize, 16 + len(body)) + body


def chunk(raw: bytes, comp: int, blosc: str = "lz4", zip_raw: bool = False) -> bytes:
    if comp & 4:
        frame = blosc_frame(raw, blosc)
        return struct.pack("<q", len(frame)) + frame
    if comp & 1:
        if zip_raw:
            return struct.pack("<q", -len(raw)) + raw
        z = zlib.compress(raw)
        return struct.pack("<q", len(z)) + z
    return raw


def _mask_bytes(bits):
    return np.packbits(np.asarray(bits, bool), bitorder="little").tobytes()


def values_block(vals, vmask, cmask, bg, comp, half, opts):
    """writeCompressedValues: the metadata byte, inactive values, selection mask and values."""
    vals = np.asarray(vals, np.float32)
    count = vals.size
    out = bytearray()
    bits = lambda v: np.float32(v).tobytes()
    # a half-float grid stores inactive values other than the background rounded to half
    rounded = lambda v: np.float32(np.float16(v)) if half and bits(v) != bits(bg) else np.float32(v)
    meta, inact, sel = 0, [], None
    if comp & 2 and opts.get("all_values"):
        meta = 6
    elif comp & 2:
        inactive = [v for v, a, c in zip(vals, vmask, cmask) if not a and not c]
        uniq = []
        for v in inactive:
            if all(bits(v) != bits(u) for u in uniq):
                uniq.append(v)
        nbg = -np.float32(bg)
        if not uniq or (len(uniq) == 1 and bits(uniq[0]) == bits(bg)):
            meta = 0
        elif len(uniq) == 1:
            meta, inact = (1, []) if bits(uniq[0]) == bits(nbg) else (2, [uniq[0]])
        elif len(uniq) == 2:
            a, b = uniq
            if bits(b) == bits(bg):
                a, b = b, a
            if bits(a) == bits(bg):  # selection on where the value is the background
                meta, inact = (3, []) if bits(b) == bits(nbg) else (4, [b])
                sel = np.array([bits(v) == bits(bg) for v in vals]) & ~np.asarray(vmask) & ~np.asarray(cmask)
            else:
                meta, inact = 5, [a, b]
                sel = np.array([bits(v) == bits(b) for v in vals]) & ~np.asarray(vmask) & ~np.asarray(cmask)
        else:
            meta = 6
    out += struct.pack("<b", meta)
    for v in inact:
        out += bits(rounded(v))
    if meta in (3, 4, 5):
        out += _mask_bytes(sel)
    if comp & 2 and meta != 6:
        payload = vals[np.asarray(vmask, bool)]
    else:
        payload = vals
    if half:
        if payload.size:
            out += chunk(payload.astype("<f2").tobytes(), comp, opts.get("blosc", "lz4"), opts.get("zip_raw", False))
    else:
        out += chunk(payload.astype("<f4").tobytes(), comp, opts.get("blosc", "lz4"), opts.get("zip_raw", False))
    return bytes(out)


# ---------------------------------------------------------------------- file
def _name(s: str) -> bytes:
    b = s.encode("latin-1")
    return struct.pack("<I", len(b)) + b


def _meta(entries):
    out = struct.pack("<I", len(entries))
    for name, typ, payload in entries:
        out += _name(name) + _name(typ) + struct.pack("<I", len(payload)) + payload
    return out


TRANSFORMS = {
    "UniformScaleMap": struct.pack("<15d", *([0.05] * 3 + [0.05] * 3 + [20.0] * 3 + [400.0] * 3 + [10.0] * 3)),
    "AffineMap": struct.pack("<16d", *np.eye(4).reshape(-1)),
    "ScaleTranslateMap": struct.pack("<18d", *range(18)),
    "TranslationMap": struct.pack("<3d", 1.0, 2.0, 3.0),
    "UnitaryMap": struct.pack("<16d", *np.eye(4).reshape(-1)),
    "NonlinearFrustumMap": struct.pack("<8d", *range(8)) + _name("AffineMap") + struct.pack("<16d", *range(16)),
}


def grid_bytes(g: Grid, comp: int, transform: str = "UniformScaleMap", opts=None) -> tuple:
    """(topology part, buffer part) of a grid: compression, metadata, transform, topology; then
    the leaves' buffers."""
    opts = opts or {}
    half = g.half
    head = struct.pack("<I", comp)
    head += _meta([("class", "string", b"fog volume"), ("name", "string", g.name.encode()),
                   ("file_voxel_count", "int64", struct.pack("<q", 12345))])
    head += _name(transform) + TRANSFORMS[transform]
    head += struct.pack("<i", 1) + g.background.tobytes()
    nodes5 = g._nodes5()
    tiles = [(o, v, a) for o, (v, a) in sorted(g.root_tiles.items()) if o not in nodes5]
    head += struct.pack("<II", len(tiles), len(nodes5))
    for o, v, a in tiles:
        head += struct.pack("<iiifB", *o, v, 1 if a else 0)
    nodes4 = set(g._nodes4())
    buffers = b""
    for o5 in nodes5:
        head += struct.pack("<iii", *o5)
        cm, vm = np.zeros(32768, bool), np.zeros(32768, bool)
        vals = np.full(32768, g.background, np.float32)
        kids = []
        for i in range(32768):
            o = (o5[0] + ((i >> 10) << 7), o5[1] + (((i >> 5) & 31) << 7), o5[2] + ((i & 31) << 7))
            if o in nodes4:
                cm[i] = True
                vals[i] = 0.0
                kids.append(o)
            elif o in g.tiles128:
                vals[i], vm[i] = g.tiles128[o][0], g.tiles128[o][1]
        head += _mask_bytes(cm) + _mask_bytes(vm) + values_block(vals, vm, cm, g.background, comp, half, opts)
        for o4 in kids:
            cm4, vm4 = np.zeros(4096, bool), np.zeros(4096, bool)
            vals4 = np.full(4096, g.background, np.float32)
            leaves = []
            for j in range(4096):
                o = (o4[0] + ((j >> 8) << 3), o4[1] + (((j >> 4) & 15) << 3), o4[2] + ((j & 15) << 3))
                if o in g.leaves:
                    cm4[j] = True
                    vals4[j] = 0.0
                    leaves.append(o)
                elif o in g.tiles8:
                    vals4[j], vm4[j] = g.tiles8[o][0], g.tiles8[o][1]
            head += _mask_bytes(cm4) + _mask_bytes(vm4) + values_block(vals4, vm4, cm4, g.background, comp, half, opts)
            for ol in leaves:
                lv, la = g.leaves[ol]
                head += _mask_bytes(la)
                buffers += _mask_bytes(la) + values_block(lv, la, np.zeros(512, bool), g.background, comp, half, opts)
    return head, buffers


def vdb_file(grids, offsets=True, version=224, comp=3, transform="UniformScaleMap", opts=None,
             extra_types=None) -> bytes:
    """A file holding `grids` in order; extra_types maps a grid's index to a grid type other than
    float (its body is then filler bytes: a reader must skip it by its end position)."""
    extra_types = extra_types or {}
    out = bytearray()
    out += struct.pack("<qIIIB", MAGIC, version, 6, 2, 1 if offsets else 0)
    out += b"0123abcd-0000-4000-8000-0123456789ab"
    out += _meta([("creator", "string", b"tests/vdb_writer.py")])
    out += struct.pack("<i", len(grids))
    for k, g in enumerate(grids):
        kind = extra_types.get(k, "Tree_float_5_4_3")
        out += _name(g.name + ("\x1e" + str(k) if k else "")) + _name(kind + ("_HalfFloat" if g.half else "")) + \
            _name("")
        pos_at = len(out)
        out += struct.pack("<qqq", 0, 0, 0)
        grid_pos = len(out)
        if kind != "Tree_float_5_4_3":
            body = b"\xee" * 40
            out += body
            block_pos = end_pos = len(out)
        else:
            head, buffers = grid_bytes(g, comp, transform, opts)
            out += head
            block_pos = len(out)
            out += buffers
            end_pos = len(out)
        if offsets:
            out[pos_at:pos_at + 24] = struct.pack("<qqq", grid_pos, block_pos, end_pos)
    return bytes(out)
