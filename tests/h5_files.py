"""Byte-level HDF5 files for the tests, written from the HDF5 file format specification.

libhdf5 / h5py are not available where the tests run, so this module lays files out
the way libhdf5 does for the two formats a user's files come in:

* ``earliest`` (libhdf5's default, what h5py writes unless told otherwise): superblock
  version 0, version 1 object headers, groups as a symbol table -- a v1 B-tree of
  symbol table nodes (SNOD) with names in a local heap whose free space is a free
  block -- datasets with a modification time message and NIL padding, raw data from
  2048 bytes on;
* ``latest`` (libver='latest'): superblock version 2 and version 2 object headers
  ("OHDR", Jenkins lookup3 checksums), groups as link info + group info + link
  messages, fill value version 3.

Datasets may be contiguous, compact or chunked (v1 B-tree chunk index, edge chunks
padded), in either byte order, and headers may continue in a second block.  The
module also reads back the int64 label datasets the library writes (``read_labels``)
and checks their structure (``check_structure``): every block in the file, no two
overlapping, the end-of-file address, sorted symbol table nodes and B-tree keys that
bound them.  It shares no code with the library's C++ implementation.
"""
from __future__ import annotations

import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIG = b"\x89HDF\r\n\x1a\n"


# ----------------------------------------------------------------- checksums

def lookup3(data: bytes, initval: int = 0) -> int:
    """Bob Jenkins' lookup3 hashlittle (the checksum of the HDF5 1.8+ structures)."""
    M = 0xFFFFFFFF

    def rot(x, k):
        return ((x << k) | (x >> (32 - k))) & M

    length = len(data)
    a = b = c = (0xDEADBEEF + length + initval) & M
    i = 0
    while length > 12:
        a = (a + int.from_bytes(data[i:i + 4], "little")) & M
        b = (b + int.from_bytes(data[i + 4:i + 8], "little")) & M
        c = (c + int.from_bytes(data[i + 8:i + 12], "little")) & M
        a = (a - c) & M; a ^= rot(c, 4); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 6); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 8); b = (b + a) & M
        a = (a - c) & M; a ^= rot(c, 16); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 19); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 4); b = (b + a) & M
        i += 12
        length -= 12
    if length == 0:
        return c
    tail = data[i:] + b"\0" * (12 - length)
    a = (a + int.from_bytes(tail[0:4], "little")) & M
    b = (b + int.from_bytes(tail[4:8], "little")) & M
    c = (c + int.from_bytes(tail[8:12], "little")) & M
    c ^= b; c = (c - rot(b, 14)) & M
    a ^= c; a = (a - rot(c, 11)) & M
    b ^= a; b = (b - rot(a, 25)) & M
    c ^= b; c = (c - rot(b, 16)) & M
    a ^= c; a = (a - rot(c, 4)) & M
    b ^= a; b = (b - rot(a, 14)) & M
    c ^= b; c = (c - rot(b, 24)) & M
    return c


# ----------------------------------------------------------------- messages

def q(v):
    return struct.pack("<Q", v)


def dt_fixed(size, signed, big=False, precision=None, offset=0):
    flags = (1 if big else 0) | (8 if signed else 0)
    return bytes([0x10, flags, 0, 0]) + struct.pack("<IHH", size, offset, size * 8 if precision is None else precision)


_FLOAT = {2: (15, 10, 5, 10, 15), 4: (31, 23, 8, 23, 127), 8: (63, 52, 11, 52, 1023)}


def dt_float(size, big=False):
    sign, eloc, esize, msize, bias = _FLOAT[size]
    flags = (1 if big else 0) | (2 << 4)  # implied leading mantissa bit
    return bytes([0x11, flags, sign, 0]) + struct.pack("<IHHBBBBI", size, 0, size * 8, eloc, esize, 0, msize, bias)


def dt_string(size):
    return bytes([0x13, 0, 0, 0]) + struct.pack("<I", size)


def dtype_message(dt: np.dtype, big=False):
    dt = np.dtype(dt)
    if dt.kind == "f":
        return dt_float(dt.itemsize, big)
    return dt_fixed(dt.itemsize, dt.kind == "i", big)


def space_v1(dims, maxdims=True):
    body = bytes([1, len(dims), 1 if maxdims else 0, 0, 0, 0, 0, 0]) + b"".join(q(d) for d in dims)
    return body + (b"".join(q(d) for d in dims) if maxdims else b"")


def space_v2(dims):
    return bytes([2, len(dims), 0, 1]) + b"".join(q(d) for d in dims)


def fill_v2(value: bytes | None = None):
    if value is None:
        return bytes([2, 2, 2, 0])
    return bytes([2, 2, 2, 1]) + struct.pack("<I", len(value)) + value


def fill_v3(value: bytes | None = None):
    if value is None:
        return bytes([3, 0x0A])  # late allocation, fill written if set, undefined
    return bytes([3, 0x2A]) + struct.pack("<I", len(value)) + value


def layout_contiguous(addr, size):
    return bytes([3, 1]) + q(addr) + q(size)


def layout_compact(raw: bytes):
    return bytes([3, 0]) + struct.pack("<H", len(raw)) + raw


def layout_chunked(btree, chunk, elsize):
    return bytes([3, 2, len(chunk) + 1]) + q(btree) + b"".join(struct.pack("<I", c) for c in list(chunk) + [elsize])


def mtime():
    return bytes([1, 0, 0, 0]) + struct.pack("<I", 1_700_000_000)


# ----------------------------------------------------------------- file builder

class H5:
    """A file under construction; addresses are absolute (base address 0)."""

    def __init__(self, fmt="earliest", leaf_k=4, internal_k=16):
        self.fmt = fmt
        self.leaf_k, self.internal_k = leaf_k, internal_k
        self.b = bytearray(104 if fmt == "earliest" else 48)  # room for a version 1 superblock

    def alloc(self, n, align=8):
        a = (len(self.b) + align - 1) // align * align
        self.b.extend(b"\0" * (a + n - len(self.b)))
        return a

    def put(self, addr, data):
        self.b[addr:addr + len(data)] = data

    def raw(self, data: bytes, at=None):
        if at is not None and at >= len(self.b):
            self.alloc(at - len(self.b), 1)
        a = self.alloc(len(data))
        self.put(a, data)
        return a

    # -- object headers
    def header_v1(self, msgs, split=None, pad=0):
        """msgs: [(type, flags, body)]; split: index where a continuation block starts."""
        def block(ms):
            out = bytearray()
            for t, fl, body in ms:
                size = (len(body) + 7) // 8 * 8
                out += struct.pack("<HHB3x", t, size, fl) + body + b"\0" * (size - len(body))
            return out
        first, second = (msgs, []) if split is None else (msgs[:split], msgs[split:])
        nmsg = len(msgs) + (1 if second else 0) + (1 if pad else 0)
        a = self.alloc(16 + len(block(first)) + (24 if second else 0) + (8 + pad if pad else 0))
        body = block(first)
        if second:
            cont_body = block(second)
            ca = self.alloc(len(cont_body))
            self.put(ca, cont_body)
            body += block([(0x10, 0, q(ca) + q(len(cont_body)))])
        if pad:
            body += block([(0x00, 0, b"\0" * pad)])  # NIL message: free space in the header
        self.put(a, struct.pack("<BBHII4x", 1, 0, nmsg, 1, len(body)) + body)
        return a

    def header_v2(self, msgs, split=None, hflags=0x02):
        """hflags: bits 0-1 width of the chunk-size field, 0x04 creation order tracked
        (two more bytes per message header), 0x10 attribute phase change values, 0x20
        access/modification/change/birth times."""
        order = bool(hflags & 0x04)

        def block(ms):
            out = b""
            for i, (t, fl, body) in enumerate(ms):
                out += struct.pack("<BHB", t, len(body), fl) + (struct.pack("<H", i) if order else b"") + body
            return out
        first, second = (msgs, []) if split is None else (msgs[:split], msgs[split:])
        body0 = block(first)
        cont_len = (4 + (2 if order else 0) + 16) if second else 0
        size0 = len(body0) + cont_len
        width = 1 << (hflags & 3)
        prefix = b"OHDR" + bytes([2, hflags])
        if hflags & 0x20:
            prefix += struct.pack("<IIII", 1_700_000_000, 1_700_000_001, 1_700_000_002, 1_700_000_003)
        if hflags & 0x10:
            prefix += struct.pack("<HH", 8, 6)
        prefix += size0.to_bytes(width, "little")
        a = self.alloc(len(prefix) + size0 + 4)
        if second:
            cont = b"OCHK" + block(second)
            cont += struct.pack("<I", lookup3(cont))
            ca = self.raw(cont)
            body0 += block([(0x10, 0, q(ca) + q(len(cont)))])
        head = prefix + body0
        self.put(a, head + struct.pack("<I", lookup3(head)))
        return a

    def header(self, msgs, split=None, pad=0, hflags=0x02):
        if self.fmt == "earliest":
            return self.header_v1(msgs, split, pad)
        return self.header_v2(msgs, split, hflags)

    # -- datasets
    def dataset(self, arr: np.ndarray, layout="contiguous", big=False, chunk=None, fill=None, split=None,
                unwritten=False, dtype_msg=None, space=None, extra=(), chunks_per_node=None, layout_version=3,
                fill_style="new", hflags=0x02):
        arr = np.ascontiguousarray(arr)
        dt = arr.dtype.newbyteorder(">" if big else "<")
        raw = arr.astype(dt).tobytes()
        es = arr.dtype.itemsize
        dims = arr.shape
        dims_es = b"".join(struct.pack("<I", x) for x in list(dims) + [es])
        if layout == "contiguous":
            addr = UNDEF if unwritten else self.raw(raw, at=2048 if self.fmt == "earliest" and len(self.b) < 2048 else None)
            lay = layout_contiguous(addr, len(raw))
            if layout_version < 3:  # versions 1 and 2: dimensions with the element size last
                lay = bytes([layout_version, len(dims) + 1, 1, 0, 0, 0, 0, 0]) + q(addr) + dims_es
        elif layout == "compact":
            lay = layout_compact(raw)
            if layout_version < 3:
                lay = (bytes([layout_version, len(dims) + 1, 0, 0, 0, 0, 0, 0]) + dims_es +
                       struct.pack("<I", len(raw)) + raw)
        else:
            btree = UNDEF if unwritten else self.chunk_btree(arr.astype(dt), chunk, chunks_per_node)
            lay = layout_chunked(btree, chunk, es)
            if layout_version < 3:
                lay = (bytes([layout_version, len(dims) + 1, 2, 0, 0, 0, 0, 0]) + q(btree) +
                       b"".join(struct.pack("<I", c) for c in list(chunk) + [es]))
        if fill_style == "old":  # fill value message of the 1.4 format: size, value
            fillmsg = (0x04, 1, struct.pack("<I", len(fill or b"")) + (fill or b""))
        elif fill_style == "v1":  # version 1: the size is always present
            fillmsg = (0x05, 1, bytes([1, 2, 2, 1 if fill else 0]) + struct.pack("<I", len(fill or b"")) + (fill or b""))
        else:
            fillmsg = (0x05, 1, (fill_v2 if self.fmt == "earliest" else fill_v3)(fill))
        msgs = [(0x01, 0, space or (space_v1 if self.fmt == "earliest" else space_v2)(dims)),
                (0x03, 1, dtype_msg or dtype_message(arr.dtype, big)), fillmsg, (0x08, 0, lay)]
        msgs += list(extra)
        if self.fmt == "earliest":
            msgs.append((0x12, 0, mtime()))
        return self.header(msgs, split, pad=136 if self.fmt == "earliest" else 0, hflags=hflags)

    def chunk_btree(self, arr, chunk, per_node=None):
        """v1 B-tree (type 1) over the chunks of arr, edge chunks padded; two levels when
        per_node is given and there are more chunks than that."""
        rank = arr.ndim
        es = arr.dtype.itemsize
        grid = [range(0, arr.shape[k], chunk[k]) for k in range(rank)]
        entries = []
        for origin in np.array(np.meshgrid(*grid, indexing="ij")).reshape(rank, -1).T:
            block = np.zeros(chunk, dtype=arr.dtype)
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(origin, chunk, arr.shape))
            block[tuple(slice(0, s.stop - s.start) for s in sl)] = arr[sl]
            entries.append((tuple(int(o) for o in origin), self.raw(block.tobytes())))
        key = lambda origin: struct.pack("<II", int(np.prod(chunk)) * es, 0) + b"".join(q(o) for o in origin) + q(0)

        def node(level, items):  # items: (origin, child address)
            body = b"TREE" + bytes([1, level]) + struct.pack("<H", len(items)) + q(UNDEF) + q(UNDEF)
            for origin, child in items:
                body += key(origin) + q(child)
            body += key(tuple(s for s in arr.shape))  # right-most key: past the last chunk
            return self.raw(body)

        if per_node is None or len(entries) <= per_node:
            return node(0, entries)
        leaves = [entries[i:i + per_node] for i in range(0, len(entries), per_node)]
        return node(1, [(lv[0][0], node(0, lv)) for lv in leaves])

    # -- groups
    def symbol_table_group(self, children: dict, snod_size=None, levels=1):
        """Group B-tree + local heap + SNODs for {name: header address}; returns (btree, heap)."""
        names = sorted(children, key=lambda s: s.encode())
        heap_data = bytearray(8)
        offs = {}
        for nm in names:
            offs[nm] = len(heap_data)
            enc = nm.encode() + b"\0"
            heap_data += enc + b"\0" * ((8 - len(enc) % 8) % 8)
        free_at = len(heap_data)
        heap_data += struct.pack("<QQ", 1, 24) + b"\0" * 8  # one free block of 24 bytes, end of list
        heap = self.alloc(32)
        seg = self.raw(bytes(heap_data))
        self.put(heap, b"HEAP" + bytes([0, 0, 0, 0]) + q(len(heap_data)) + q(free_at) + q(seg))
        per = snod_size or 2 * self.leaf_k
        snods = []
        for i in range(0, len(names), per):
            part = names[i:i + per]
            a = self.alloc(8 + 2 * self.leaf_k * 40)
            body = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(part))
            for nm in part:
                body += q(offs[nm]) + q(children[nm]) + struct.pack("<II", 0, 0) + b"\0" * 16
            self.put(a, body)
            snods.append((part[-1], a))
        node_size = 24 + 2 * self.internal_k * 8 + (2 * self.internal_k + 1) * 8

        def node(level, items):  # items: (largest name below, child)
            a = self.alloc(node_size)
            body = b"TREE" + bytes([0, level]) + struct.pack("<H", len(items)) + q(UNDEF) + q(UNDEF) + q(0)
            for last, child in items:
                body += q(child) + q(offs[last])
            self.put(a, body)
            return a

        if levels == 1 or len(snods) < 2:
            return node(0, snods), heap
        half = (len(snods) + 1) // 2
        left, right = node(0, snods[:half]), node(0, snods[half:])
        return node(1, [(snods[half - 1][0], left), (snods[-1][0], right)]), heap

    def group(self, children: dict, link_flags=0x00, dense=False, **kw):
        """A group object of this file's format holding {name: header address}.
        link_flags (latest format): 0x08 link type stored, 0x04 creation order stored,
        0x10 character set stored; dense: the link info names a fractal heap (dense
        link storage), which this module does not write out."""
        if self.fmt == "earliest":
            bt, hp = self.symbol_table_group(children, **kw)
            return self.header_v1([(0x11, 0, q(bt) + q(hp))]), (bt, hp)
        msgs = [(0x02, 0, bytes([0, 0]) + q(4096 if dense else UNDEF) + q(UNDEF)), (0x0A, 0, bytes([0, 0]))]
        for i, (nm, addr) in enumerate(children.items()):
            enc = nm.encode()
            body = bytes([1, link_flags])
            if link_flags & 0x08:
                body += bytes([0])  # hard link
            if link_flags & 0x04:
                body += q(i)
            if link_flags & 0x10:
                body += bytes([1])  # UTF-8
            body += bytes([len(enc)]) + enc + q(addr)
            msgs.append((0x06, 0, body))
        return self.header_v2(msgs), None

    def finish(self, root_children: dict, path, sb_version=None, **kw):
        root, st = self.group(root_children, **kw)
        eof = len(self.b)
        if self.fmt == "earliest":
            bt, hp = st
            v = sb_version or 0
            sb = SIG + bytes([v, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", self.leaf_k, self.internal_k, 0)
            if v == 1:  # indexed storage internal node K, reserved
                sb += struct.pack("<HH", 32, 0)
            sb += q(0) + q(UNDEF) + q(eof) + q(UNDEF)
            sb += q(0) + q(root) + struct.pack("<II", 1, 0) + q(bt) + q(hp)
        else:
            sb = SIG + bytes([2, 8, 8, 0]) + q(0) + q(UNDEF) + q(eof) + q(root)
            sb += struct.pack("<I", lookup3(sb))
        self.put(0, sb)
        with open(path, "wb") as f:
            f.write(bytes(self.b))


def write_matrix(path, arr, name="DATA", fmt="earliest", **kw):
    """A file holding one 2-D dataset `name` (inside groups for a path 'a/b/name')."""
    f = H5(fmt)
    parts = name.strip("/").split("/")
    child = {parts[-1]: f.dataset(arr, **kw)}
    for g in reversed(parts[:-1]):
        gaddr, _ = f.group(child)
        child = {g: gaddr}
    f.finish(child, path)


# ----------------------------------------------------------------- reading back

class Reader:
    """Independent reader of symbol-table files written by the library."""

    def __init__(self, path):
        with open(path, "rb") as fh:
            raw = fh.read()
        sb = next(a for a in (0, 512, 1024, 2048, 4096) if raw[a:a + 8] == SIG)
        assert raw[sb + 8] == 0, "superblock version"
        self.file_size = len(raw)
        self.eof = struct.unpack_from("<Q", raw, sb + 40)[0]  # counts from the start of the file
        base = struct.unpack_from("<Q", raw, sb + 24)[0]
        self.b = raw[base:]  # addresses below are relative to the base address
        self.root = struct.unpack_from("<Q", raw, sb + 64)[0]
        assert struct.unpack_from("<I", raw, sb + 72)[0] == 1
        self.root_bt, self.root_heap = struct.unpack_from("<QQ", raw, sb + 80)
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", raw, sb + 16)
        self.blocks = [(sb - base, 96, "superblock")] if sb >= base else []

    def u64(self, a):
        return struct.unpack_from("<Q", self.b, a)[0]

    def heap(self, a):
        assert self.b[a:a + 4] == b"HEAP"
        size, free, data = struct.unpack_from("<QQQ", self.b, a + 8)
        assert free == 1 or (free % 8 == 0 and free < size), "free list head"
        return size, data

    def name(self, heap, off):
        size, data = heap
        end = self.b.index(b"\0", data + off)
        assert end < data + size
        return self.b[data + off:end].decode()

    def group_entries(self, bt, heap_addr, record=False):
        heap = self.heap(heap_addr)
        if record:
            self.blocks += [(heap_addr, 32, "heap"), (heap[1], heap[0], "heap data")]
        out = []
        node_size = 24 + 2 * self.internal_k * 8 + (2 * self.internal_k + 1) * 8

        def walk(a, lo, hi):
            assert self.b[a:a + 4] == b"TREE" and self.b[a + 4] == 0
            if record:
                self.blocks.append((a, node_size, "group B-tree"))
            level, used = self.b[a + 5], struct.unpack_from("<H", self.b, a + 6)[0]
            assert 0 < used <= 2 * self.internal_k
            keys = [self.u64(a + 24 + 16 * i) for i in range(used + 1)]
            kids = [self.u64(a + 32 + 16 * i) for i in range(used)]
            for i, c in enumerate(kids):
                klo = self.name(heap, keys[i]) if i else lo
                khi = self.name(heap, keys[i + 1])
                if level:
                    walk(c, klo, khi)
                    continue
                assert self.b[c:c + 4] == b"SNOD"
                if record:
                    self.blocks.append((c, 8 + 2 * self.leaf_k * 40, "SNOD"))
                n = struct.unpack_from("<H", self.b, c + 6)[0]
                assert 0 < n <= 2 * self.leaf_k
                names = []
                for k in range(n):
                    e = c + 8 + 40 * k
                    nm = self.name(heap, self.u64(e))
                    names.append(nm)
                    out.append((nm, self.u64(e + 8)))
                enc = [s.encode() for s in names]
                assert enc == sorted(enc), "SNOD entries out of order"
                assert enc[-1] <= khi.encode(), "B-tree key below a name of its child"
                if klo is not None and i:
                    assert enc[0] > klo.encode(), "B-tree key above a name of the next child"

        walk(bt, None, None)
        return out

    def labels(self, name, record=False, record_group=False):
        ents = dict(self.group_entries(self.root_bt, self.root_heap, record_group))
        h = ents[name]
        assert self.b[h] == 1, "object header version"
        nmsg, _, hsize = struct.unpack_from("<HII", self.b, h + 2)
        assert hsize % 8 == 0
        if record:
            self.blocks.append((h, 16 + hsize, "dataset header " + name))
        a, seen, dims, layout, dtype = h + 16, 0, None, None, None
        while seen < nmsg:
            t, size, _fl = struct.unpack_from("<HHB", self.b, a)
            assert size % 8 == 0
            body = self.b[a + 8:a + 8 + size]
            if t == 0x01:
                rank = body[1]
                dims = struct.unpack_from("<%dQ" % rank, body, 8)
            elif t == 0x03:
                dtype = body[:12]
            elif t == 0x08:
                assert body[0] == 3 and body[1] == 1
                layout = struct.unpack_from("<QQ", body, 2)
            a += 8 + size
            seen += 1
        assert a == h + 16 + hsize
        assert dtype == bytes([0x10, 0x08, 0, 0, 8, 0, 0, 0, 0, 0, 64, 0]), "int64 little-endian"
        n = dims[0]
        addr, size = layout
        assert size == 8 * n
        if n == 0:
            return np.zeros(0, np.int64)
        if record:
            self.blocks.append((addr, size, "data " + name))
        return np.frombuffer(self.b, dtype="<i8", count=n, offset=addr).copy()


def read_labels(path, name):
    return Reader(path).labels(name)


def check_structure(path, names):
    """Every block the library's writer placed, within the end-of-file address and
    without overlaps; returns the labels of each dataset."""
    r = Reader(path)
    assert r.eof == r.file_size, "end-of-file address differs from the file size"
    r.blocks.append((r.root, 16 + struct.unpack_from("<I", r.b, r.root + 8)[0], "root header"))
    out = {}
    for i, nm in enumerate(names):
        out[nm] = r.labels(nm, record=True, record_group=(i == 0))
    blocks = sorted(r.blocks)
    for (a0, s0, n0), (a1, s1, n1) in zip(blocks, blocks[1:]):
        assert a0 + s0 <= a1, f"{n0} at {a0}+{s0} overlaps {n1} at {a1}"
    assert blocks[-1][0] + blocks[-1][1] <= len(r.b)
    return out
