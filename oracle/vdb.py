"""OpenVDB density grids for the oracle's scene reader.

TEST INFRASTRUCTURE: imported only by oracle/scene_reader.py (itself only used by tests/,
__graft_entry__.smoke() and bench.py's CPU legs). The product never imports it.

Restates core/ResourceManager.cpp:165-218 (loadVDBasTexture) over the file layout of OpenVDB 6.2,
the library the reference links (includes/openvdb: io/Archive.cc readHeader, io/GridDescriptor.cc
read, MetaMap.cc readMeta, math/Transform.cc and math/Maps.h read, tree/RootNode.h,
InternalNode.h and LeafNode.h readTopology / readBuffers, io/Compression.h readCompressedValues,
io/Compression.cc unzipFromStream / bloscFromStream, tools/Dense.h copyToDense with the
LayoutZYX array), with the public Blosc-1 frame and LZ4 block formats. Written independently of
the library's reader (narvalengine_gb300/csrc/vdb_read.cpp): here the dense array is formed
voxel by voxel through a lookup in the tree, as copyToDense reads the tree, where the library
paints each node over its part of the box.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

MAGIC = 0x56444220
ZIP, ACTIVE_MASK, BLOSC = 1, 2, 4


class VdbError(Exception):
    """`kind` is "parse", "unsupported" or "missing"."""

    def __init__(self, kind, msg):
        super().__init__(msg)
        self.kind = kind


class _Stream:
    def __init__(self, data):
        self.b = data
        self.pos = 0

    def take(self, n):
        if n < 0 or self.pos + n > len(self.b):
            raise VdbError("parse", "truncated file")
        out = self.b[self.pos:self.pos + n]
        self.pos += n
        return out

    def unpack(self, fmt):
        return struct.unpack("<" + fmt, self.take(struct.calcsize("<" + fmt)))

    def name(self):
        (n,) = self.unpack("I")
        return self.take(n).decode("latin-1")


def _mask(st, bits):
    return np.unpackbits(np.frombuffer(st.take(bits // 8), np.uint8), bitorder="little").astype(bool)


def _lz4(src, size):
    out = bytearray()
    i = 0
    while i < len(src):
        token = src[i]
        i += 1
        lit = token >> 4
        if lit == 15:
            while True:
                if i >= len(src):
                    raise VdbError("parse", "truncated LZ4 stream")
                lit += src[i]
                i += 1
                if src[i - 1] != 255:
                    break
        if i + lit > len(src):
            raise VdbError("parse", "corrupt LZ4 literals")
        out += src[i:i + lit]
        i += lit
        if i >= len(src):
            break
        if i + 2 > len(src):
            raise VdbError("parse", "truncated LZ4 offset")
        off = src[i] | (src[i + 1] << 8)
        i += 2
        if off == 0 or off > len(out):
            raise VdbError("parse", "corrupt LZ4 offset")
        n = token & 15
        if n == 15:
            while True:
                if i >= len(src):
                    raise VdbError("parse", "truncated LZ4 stream")
                n += src[i]
                i += 1
                if src[i - 1] != 255:
                    break
        n += 4
        start = len(out) - off
        for k in range(n):  # the match may overlap what it copies
            out.append(out[start + k])
        if len(out) > size:
            raise VdbError("parse", "corrupt LZ4 match")
    return bytes(out)


def _blosc(frame, want):
    if len(frame) < 16:
        raise VdbError("parse", "truncated Blosc frame")
    flags, typesize = frame[2], frame[3]
    nbytes, blocksize, cbytes = struct.unpack_from("<III", frame, 4)
    if nbytes != want or cbytes > len(frame):
        raise VdbError("parse", "Blosc frame of an unexpected size")
    if flags & 0x02:  # stored as is after the header
        if 16 + nbytes > len(frame):
            raise VdbError("parse", "truncated Blosc frame")
        return frame[16:16 + nbytes]
    if flags >> 5 != 1:
        raise VdbError("unsupported", "Blosc codec other than LZ4")
    if flags & 0x04:
        raise VdbError("unsupported", "Blosc bit shuffle")
    if nbytes == 0:
        return b""
    if blocksize == 0 or blocksize > nbytes or typesize == 0:
        raise VdbError("parse", "corrupt Blosc header")
    nblocks = -(-nbytes // blocksize)
    if 16 + 4 * nblocks > len(frame):
        raise VdbError("parse", "truncated Blosc frame")
    starts = struct.unpack_from(f"<{nblocks}i", frame, 16)
    out = bytearray()
    for j in range(nblocks):
        last = j == nblocks - 1 and nbytes % blocksize != 0
        bsize = nbytes % blocksize if last else blocksize
        split = not (flags & 0x10) and typesize <= 16 and bsize // typesize >= 128 and not last
        nsplit = typesize if split else 1
        if bsize % nsplit:
            raise VdbError("parse", "corrupt Blosc block")
        neblock = bsize // nsplit
        at = starts[j]
        block = bytearray()
        for _ in range(nsplit):
            if at < 0 or at + 4 > len(frame):
                raise VdbError("parse", "truncated Blosc block")
            (cs,) = struct.unpack_from("<i", frame, at)
            at += 4
            if cs < 0 or at + cs > len(frame):
                raise VdbError("parse", "corrupt Blosc stream size")
            part = frame[at:at + cs]
            at += cs
            if cs == neblock:
                block += part
            else:
                dec = _lz4(part, neblock)
                if len(dec) != neblock:
                    raise VdbError("parse", "LZ4 stream of an unexpected size")
                block += dec
        if flags & 0x01 and typesize > 1:  # undo the byte shuffle
            count = bsize // typesize
            body = np.frombuffer(bytes(block[:count * typesize]), np.uint8).reshape(typesize, count)
            block = bytearray(body.T.tobytes()) + block[count * typesize:]
        out += block
    return bytes(out)


def _data(st, comp, nbytes):
    if not comp & (ZIP | BLOSC):
        return st.take(nbytes)
    (n,) = st.unpack("q")
    if n <= 0:
        if -n != nbytes:
            raise VdbError("parse", "raw chunk of an unexpected size")
        return st.take(nbytes)
    chunk = st.take(n)
    if comp & BLOSC:
        return _blosc(chunk, nbytes)
    try:
        out = zlib.decompress(chunk)
    except zlib.error as e:
        raise VdbError("parse", f"zip chunk: {e}")
    if len(out) != nbytes:
        raise VdbError("parse", "zip chunk of an unexpected size")
    return out


def _values(st, comp, half, bg, count, vmask):
    """readCompressedValues: float32 array of `count` values."""
    (meta,) = st.unpack("b")
    bg = np.float32(bg)
    inact1 = bg
    inact0 = bg if meta == 0 else -bg
    if meta in (2, 4, 5):
        inact0 = np.float32(st.unpack("f")[0])
        if meta == 5:
            inact1 = np.float32(st.unpack("f")[0])
    sel = _mask(st, count) if meta in (3, 4, 5) else np.zeros(count, bool)
    masked = bool(comp & ACTIVE_MASK)
    stored = int(vmask.sum()) if masked and meta != 6 else count
    if half:
        vals = np.frombuffer(_data(st, comp, 2 * stored), "<f2").astype(np.float32) if stored else \
            np.zeros(0, np.float32)
    else:
        vals = np.frombuffer(_data(st, comp, 4 * stored), "<f4").astype(np.float32)
    if masked and stored != count:
        out = np.where(sel, inact1, inact0).astype(np.float32)
        out[vmask] = vals
        return out
    return vals.copy()


def _skip_meta(st):
    (count,) = st.unpack("I")
    for _ in range(count):
        st.name()
        st.name()
        (n,) = st.unpack("I")
        st.take(n)


_MAP_DOUBLES = {"AffineMap": 16, "UnitaryMap": 16, "ScaleMap": 15, "UniformScaleMap": 15, "TranslationMap": 3,
                "ScaleTranslateMap": 18, "UniformScaleTranslateMap": 18}


def _skip_map(st, kind, nested=False):
    if kind in _MAP_DOUBLES:
        st.take(8 * _MAP_DOUBLES[kind])
    elif kind == "NonlinearFrustumMap" and not nested:
        st.take(8 * 8)
        _skip_map(st, st.name(), True)
    else:
        raise VdbError("unsupported", f"VDB transform {kind}")


class _Node:
    """An internal node (log2 5 or 4): child and value masks, values, children by offset."""

    def __init__(self, origin, log2):
        low = (1 << (12 if log2 == 5 else 7)) - 1
        self.origin = tuple(c & ~low for c in origin)
        self.log2 = log2
        self.children = {}


def _child_origin(origin, i, log2, shift):
    m = (1 << log2) - 1
    return (origin[0] + ((i >> (2 * log2)) << shift), origin[1] + (((i >> log2) & m) << shift),
            origin[2] + ((i & m) << shift))


def _read_node(st, comp, half, bg, origin, log2):
    size = 1 << (3 * log2)
    nd = _Node(origin, log2)
    nd.cmask = _mask(st, size)
    nd.vmask = _mask(st, size)
    nd.values = _values(st, comp, half, bg, size, nd.vmask)
    for i in np.nonzero(nd.cmask)[0]:
        i = int(i)
        if log2 == 5:
            nd.children[i] = _read_node(st, comp, half, bg, _child_origin(nd.origin, i, 5, 7), 4)
        else:
            leaf = {"origin": _child_origin(nd.origin, i, 4, 3), "vmask": _mask(st, 512), "values": None}
            nd.children[i] = leaf
    return nd


def _read_grid(st, half):
    (comp,) = st.unpack("I")
    _skip_meta(st)
    _skip_map(st, st.name())
    st.unpack("i")  # buffer count
    (bg,) = st.unpack("f")
    ntiles, nchildren = st.unpack("II")
    root = {}
    for _ in range(ntiles):
        x, y, z, v, a = st.unpack("iiifB")
        root[(x, y, z)] = ("tile", np.float32(v), a != 0)
    for _ in range(nchildren):
        key = st.unpack("iii")
        root[key] = ("node", _read_node(st, comp, half, bg, key, 5))
    for key in sorted(root):  # RootNode::readBuffers: the table in coordinate order
        if root[key][0] != "node":
            continue
        n5 = root[key][1]
        for i in sorted(n5.children):
            n4 = n5.children[i]
            for j in sorted(n4.children):
                leaf = n4.children[j]
                st.take(64)
                leaf["values"] = _values(st, comp, half, bg, 512, leaf["vmask"])
    return np.float32(bg), root


def _active_box(root):
    lo, hi = [None] * 3, [None] * 3

    def grow(p, dim):
        for a in range(3):
            lo[a] = p[a] if lo[a] is None else min(lo[a], p[a])
            hi[a] = p[a] + dim - 1 if hi[a] is None else max(hi[a], p[a] + dim - 1)

    for key, e in root.items():
        if e[0] == "tile":
            if e[2]:
                grow(key, 4096)
            continue
        n5 = e[1]
        for i in np.nonzero(n5.vmask & ~n5.cmask)[0]:
            grow(_child_origin(n5.origin, int(i), 5, 7), 128)
        for n4 in n5.children.values():
            for j in np.nonzero(n4.vmask & ~n4.cmask)[0]:
                grow(_child_origin(n4.origin, int(j), 4, 3), 8)
            for leaf in n4.children.values():
                for k in np.nonzero(leaf["vmask"])[0]:
                    grow(_child_origin(leaf["origin"], int(k), 3, 0), 1)
    return lo, hi


def _lookup(bg, root, x, y, z):
    e = root.get((x & ~4095, y & ~4095, z & ~4095))
    if e is None:
        return bg
    if e[0] == "tile":
        return e[1]
    n5 = e[1]
    i = (((x & 4095) >> 7) << 10) | (((y & 4095) >> 7) << 5) | ((z & 4095) >> 7)
    n4 = n5.children.get(i)
    if n4 is None:
        return n5.values[i]
    j = (((x & 127) >> 3) << 8) | (((y & 127) >> 3) << 4) | ((z & 127) >> 3)
    leaf = n4.children.get(j)
    if leaf is None:
        return n4.values[j]
    return leaf["values"][((x & 7) << 6) | ((y & 7) << 3) | (z & 7)]


def load_density(path):
    """([width, height, depth] = [dim z, dim y, dim x], float32 array z fastest) of the first grid
    named "density", as loadVDBasTexture hands it to the texture."""
    try:
        data = open(path, "rb").read()
    except OSError:
        raise VdbError("missing", f"Couldn't read the file at {path}.")
    st = _Stream(data)
    (magic,) = st.unpack("q")
    if magic != MAGIC:
        raise VdbError("parse", "not a VDB file")
    (version,) = st.unpack("I")
    if version < 222:
        raise VdbError("unsupported", f"VDB file format {version} (before 222)")
    st.take(8)
    (offsets,) = st.unpack("B")
    st.take(36)
    _skip_meta(st)
    (count,) = st.unpack("i")
    for _ in range(count):
        unique, kind, parent = st.name(), st.name(), st.name()
        grid_pos, _block, end_pos = st.unpack("qqq")
        name = unique.split("\x1e")[0]
        half = kind.endswith("_HalfFloat")
        if half:
            kind = kind[:-len("_HalfFloat")]
        is_float = kind == "Tree_float_5_4_3"
        if name != "density":
            if offsets:
                if end_pos < 0 or end_pos > len(data):
                    raise VdbError("parse", "stream position outside the file")
                st.pos = end_pos
            elif is_float and not parent:
                _read_grid(st, half)
            else:
                raise VdbError("unsupported", f"VDB stream without grid offsets holding a {kind} grid")
            continue
        if not is_float:
            raise VdbError("unsupported", f"density grid of type {kind} (not a float grid)")
        if parent:
            raise VdbError("unsupported", f"density grid instanced from {parent}")
        if offsets:
            if grid_pos < 0 or grid_pos > len(data):
                raise VdbError("parse", "stream position outside the file")
            st.pos = grid_pos
        bg, root = _read_grid(st, half)
        lo, hi = _active_box(root)
        if lo[0] is None:
            raise VdbError("parse", "the density grid has no active voxels")
        dims, org = [], []
        for a in range(3):
            d = abs(lo[a]) + abs(hi[a]) + (1 if lo[a] < 0 <= hi[a] else 0)
            if d <= 0:
                raise VdbError("parse", "the dense box of the density grid is empty")
            dims.append(d)
            org.append(-abs(lo[a]))
        if 4 * dims[0] * dims[1] * dims[2] > 2 ** 31 - 1:
            raise VdbError("unsupported", "dense density grid of 2 GiB or more")
        dense = np.empty(dims, np.float32)  # [x][y][z]: LayoutZYX
        for x in range(dims[0]):
            for y in range(dims[1]):
                for z in range(dims[2]):
                    dense[x, y, z] = _lookup(bg, root, org[0] + x, org[1] + y, org[2] + z)
        return [dims[2], dims[1], dims[0]], dense.reshape(-1)
    raise VdbError("parse", "no grid named density")
