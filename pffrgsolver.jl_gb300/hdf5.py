"""A small HDF5 reader/writer for the reference's observable and checkpoint files.

The reference writes its ``*_obs`` and ``*_cp`` files with HDF5.jl (libhdf5's
default, "earliest" file format).  Neither libhdf5 nor h5py is available
here, so this module implements the subset of the HDF5 file format
specification those files use:

* superblock version 0 (8-byte offsets and lengths), with or without a user
  block in front;
* groups as symbol tables: object header (version 1) with a symbol table
  message, a version-1 B-tree of group nodes and a local heap of link names;
  B-trees of any depth in both directions, libhdf5's default node sizes
  (group leaf K = 4, internal K = 16);
* datasets with a version-1 dataspace (scalar or simple), contiguous or
  compact layout (version 3 layout message), and the datatypes HDF5.jl
  writes for the reference's values: IEEE float64, signed int64, Bool as an
  8-bit bitfield, fixed-length UTF-8 strings (the reader also takes
  variable-length strings from the global heap);
* object header continuation messages (reader).

Arrays follow HDF5.jl's convention: a Julia array of size (n1, ..., nk) is
stored with dataspace dims (nk, ..., n1) and the same bytes, so the reader
returns Fortran-ordered numpy arrays of the Julia shape.

``File(path, "cw")`` opens (or creates) a file for appending, like
``h5open(path, "cw")``: new datasets go to the end of the file, and on
``close`` the metadata of every group that gained a link is written again
after them and the superblock is pointed at the new root (the replaced
group metadata stays as unused bytes; the superblock is written last, so an
interrupted close leaves the previous state readable).  Existing datasets
and unchanged groups are never rewritten.
"""
from __future__ import annotations

import decimal
import os
import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
LEAF_K = 4       # libhdf5's defaults: symbol table nodes of 8 links,
INTERNAL_K = 16  # B-tree nodes of 32 children

# message types
MSG_NIL, MSG_DATASPACE, MSG_DATATYPE, MSG_FILL_OLD, MSG_FILL, MSG_LAYOUT = 0x0, 0x1, 0x3, 0x4, 0x5, 0x8
MSG_CONT, MSG_STAB = 0x10, 0x11


class HDF5Error(Exception):
    pass


def julia_float_str(x: float) -> str:
    """``string(x::Float64)`` of Julia (used by the reference for group names like "χ/$(Λ)"):
    shortest round-trip digits, plain notation for 1e-4 <= |x| < 1e6 (integers end in ".0"),
    otherwise "d.ddde±n" with at least one fractional digit and no exponent padding."""
    x = float(x)
    if x == 0.0:
        return "-0.0" if np.signbit(x) else "0.0"
    if not np.isfinite(x):
        return "NaN" if np.isnan(x) else ("Inf" if x > 0 else "-Inf")
    ax = abs(x)
    if 1e-4 <= ax < 1e6:
        s = repr(x)
        if "e" in s or "E" in s:  # cannot happen in this range, kept for safety
            s = format(decimal.Decimal(s), "f")
        return s if "." in s else s + ".0"
    sign, digits, exp = decimal.Decimal(repr(x)).as_tuple()
    ds = "".join(str(d) for d in digits).rstrip("0") or "0"
    e10 = exp + len(digits) - 1
    mant = ds[0] + "." + (ds[1:] if len(ds) > 1 else "0")
    return ("-" if sign else "") + mant + "e" + str(e10)


# ---------------------------------------------------------------------------
# datatypes
# ---------------------------------------------------------------------------
class _Type:
    """A parsed datatype: kind in {'f', 'i', 'u', 'b', 's', 'vs'} and element size."""

    def __init__(self, kind, size, order="<", pad=0, cset=0):
        self.kind, self.size, self.order, self.pad, self.cset = kind, size, order, pad, cset

    def numpy(self):
        if self.kind == "f":
            return np.dtype(self.order + "f%d" % self.size)
        if self.kind == "i":
            return np.dtype(self.order + "i%d" % self.size)
        if self.kind in ("u", "b"):
            return np.dtype(self.order + "u%d" % self.size)
        raise HDF5Error("no numpy type for " + self.kind)


def _parse_datatype(b: bytes) -> _Type:
    cv = b[0]
    cls, ver = cv & 0x0F, cv >> 4
    bits = b[1] | (b[2] << 8) | (b[3] << 16)
    size = struct.unpack_from("<I", b, 4)[0]
    order = ">" if bits & 1 else "<"
    if cls == 0:
        return _Type("i" if bits & 0x8 else "u", size, order)
    if cls == 1:
        return _Type("f", size, order)
    if cls == 3:
        return _Type("s", size, pad=bits & 0xF, cset=(bits >> 4) & 0xF)
    if cls == 4:
        return _Type("b", size, order)
    if cls == 9:
        vtype = bits & 0xF  # 1: string
        if vtype == 1:
            return _Type("vs", size, pad=(bits >> 4) & 0xF, cset=(bits >> 8) & 0xF)
        raise HDF5Error("variable-length sequences are not supported")
    raise HDF5Error("datatype class %d (version %d) is not supported" % (cls, ver))


def _datatype_message(value_kind: str, size: int = 8) -> bytes:
    if value_kind == "f8":  # IEEE little-endian double: implied msb, sign bit 63
        return bytes([0x11, 0x20, 63, 0]) + struct.pack("<IHHBBBBI", 8, 0, 64, 52, 11, 0, 52, 1023)
    if value_kind == "i8":  # signed little-endian 64-bit integer
        return bytes([0x10, 0x08, 0, 0]) + struct.pack("<IHH", 8, 0, 64)
    if value_kind == "b1":  # 8-bit bitfield (HDF5.jl's Bool)
        return bytes([0x14, 0, 0, 0]) + struct.pack("<IHH", 1, 0, 8)
    if value_kind == "s":  # fixed-length string, null terminated, UTF-8
        return bytes([0x13, 0x10, 0, 0]) + struct.pack("<I", size)
    raise HDF5Error(value_kind)


def _dataspace_message(dims) -> bytes:
    dims = list(dims)
    out = struct.pack("<BBBBI", 1, len(dims), 0, 0, 0)
    for d in dims:
        out += struct.pack("<Q", d)
    return out


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * ((-len(b)) % 8)


def _object_header(messages) -> bytes:
    """Version-1 object header with the given (type, data) messages (data padded to 8 bytes)."""
    body = b""
    for mtype, data in messages:
        data = _pad8(data)
        body += struct.pack("<HHB3x", mtype, len(data), 0) + data
    return struct.pack("<BBHII", 1, 0, len(messages), 1, len(body)) + b"\0" * 4 + body


# ---------------------------------------------------------------------------
# reader
# ---------------------------------------------------------------------------
class _Reader:
    def __init__(self, path):
        self.f = open(path, "rb")
        head = self.f.read(1 << 16)
        base = None
        for off in [0] + [512 << k for k in range(12)]:
            if head[off:off + 8] == SIGNATURE:
                base = off
                break
            if off >= len(head):
                self.f.seek(off)
                if self.f.read(8) == SIGNATURE:
                    base = off
                    break
        if base is None:
            raise HDF5Error("not an HDF5 file: " + str(path))
        self.f.seek(base)
        sb = self.f.read(96 + 4)
        ver = sb[8]
        if ver not in (0, 1):
            raise HDF5Error("superblock version %d is not supported (only 0 and 1)" % ver)
        if sb[13] != 8 or sb[14] != 8:
            raise HDF5Error("only 8-byte offsets and lengths are supported")
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", sb, 16)
        p = 24 + (4 if ver == 1 else 0)
        self.base_addr, _, self.eof, _ = struct.unpack_from("<QQQQ", sb, p)
        self.sb_offset = base
        self.root_entry_pos = base + p + 32
        self.root = self._entry(sb, p + 32)

    def _entry(self, b, p):
        name_off, ohdr, cache = struct.unpack_from("<QQI", b, p)
        scratch = struct.unpack_from("<QQ", b, p + 24)
        return name_off, ohdr, cache, scratch

    def read_at(self, addr, n):
        self.f.seek(self.base_addr + addr)
        return self.f.read(n)

    def messages(self, addr):
        """All messages (type, data) of the object header at addr, following continuations."""
        h = self.read_at(addr, 16)
        if h[:4] == b"OHDR":
            raise HDF5Error("version-2 object headers are not supported")
        ver, _, nmsg, _, size = struct.unpack_from("<BBHII", h, 0)
        if ver != 1:
            raise HDF5Error("object header version %d" % ver)
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            data = self.read_at(start, length)
            p = 0
            while p + 8 <= length and len(out) < nmsg:
                mtype, msize, _flags = struct.unpack_from("<HHB", data, p)
                body = data[p + 8:p + 8 + msize]
                p += 8 + msize
                if mtype == MSG_CONT:
                    caddr, clen = struct.unpack_from("<QQ", body, 0)
                    blocks.append((caddr, clen))
                out.append((mtype, body))
        return out

    def group_links(self, ohdr_addr):
        msgs = self.messages(ohdr_addr)
        stab = [m for t, m in msgs if t == MSG_STAB]
        if not stab:
            if any(t in (0x2, 0x6, 0xA) for t, _ in msgs):
                raise HDF5Error("groups with link messages (new-style groups) are not supported")
            return None
        btree, heap = struct.unpack_from("<QQ", stab[0], 0)
        names = self._heap(heap)
        links = {}
        self._walk_group_btree(btree, names, links)
        self.last_stab = (btree, heap)
        return links

    def _heap(self, addr):
        h = self.read_at(addr, 32)
        if h[:4] != b"HEAP":
            raise HDF5Error("bad local heap signature")
        size, _free, daddr = struct.unpack_from("<QQQ", h, 8)
        return self.read_at(daddr, size)

    def _walk_group_btree(self, addr, names, links):
        h = self.read_at(addr, 24)
        if h[:4] != b"TREE" or h[4] != 0:
            raise HDF5Error("bad group B-tree node")
        level = h[5]
        used = struct.unpack_from("<H", h, 6)[0]
        body = self.read_at(addr + 24, used * 16 + 8)
        children = [struct.unpack_from("<Q", body, 8 + 16 * i)[0] for i in range(used)]
        for c in children:
            if level > 0:
                self._walk_group_btree(c, names, links)
            else:
                self._snod(c, names, links)

    def _snod(self, addr, names, links):
        h = self.read_at(addr, 8)
        if h[:4] != b"SNOD":
            raise HDF5Error("bad symbol table node")
        n = struct.unpack_from("<H", h, 6)[0]
        body = self.read_at(addr + 8, 40 * n)
        for i in range(n):
            name_off, ohdr, cache, scratch = self._entry(body, 40 * i)
            end = names.index(b"\0", name_off)
            links[names[name_off:end].decode("utf-8")] = ohdr

    def dataset(self, ohdr_addr):
        dims, dtype, layout = None, None, None
        for t, m in self.messages(ohdr_addr):
            if t == MSG_DATASPACE:
                ver, rank, flags = m[0], m[1], m[2]
                p = 8 if ver == 1 else 4
                if ver == 2 and m[3] == 2:
                    dims = None  # null dataspace
                dims = [struct.unpack_from("<Q", m, p + 8 * k)[0] for k in range(rank)]
            elif t == MSG_DATATYPE:
                dtype = _parse_datatype(m)
            elif t == MSG_LAYOUT:
                layout = m
        if dtype is None or layout is None or dims is None:
            raise HDF5Error("object at %d is not a dataset" % ohdr_addr)
        n = int(np.prod(dims)) if dims else 1
        nbytes = n * dtype.size
        ver = layout[0]
        if ver == 3:
            cls = layout[1]
            if cls == 1:
                addr, size = struct.unpack_from("<QQ", layout, 2)
                raw = self.read_at(addr, size) if addr != UNDEF else b"\0" * nbytes
            elif cls == 0:
                size = struct.unpack_from("<H", layout, 2)[0]
                raw = layout[4:4 + size]
            else:
                raise HDF5Error("chunked datasets are not supported")
        elif ver in (1, 2):
            # version 1/2: dimensionality, class, 5 reserved bytes, [address], dims (4 bytes each)
            rank, cls = layout[1], layout[2]
            if cls == 1:
                addr = struct.unpack_from("<Q", layout, 8)[0]
                raw = self.read_at(addr, nbytes) if addr != UNDEF else b"\0" * nbytes
            elif cls == 0:
                p = 8 + 4 * rank
                size = struct.unpack_from("<I", layout, p)[0]
                raw = layout[p + 4:p + 4 + size]
            else:
                raise HDF5Error("chunked datasets are not supported")
        else:
            raise HDF5Error("layout message version %d is not supported" % ver)
        return self._decode(raw, dtype, dims, n)

    def _decode(self, raw, dt, dims, n):
        if dt.kind == "s":
            vals = [raw[k * dt.size:(k + 1) * dt.size].split(b"\0")[0].decode("utf-8") for k in range(n)]
            return vals[0] if not dims else np.array(vals, dtype=object).reshape(tuple(reversed(dims)), order="F")
        if dt.kind == "vs":
            vals = []
            for k in range(n):
                length, gaddr, idx = struct.unpack_from("<IQI", raw, 16 * k)
                vals.append(self._global_heap_object(gaddr, idx)[:length].decode("utf-8"))
            return vals[0] if not dims else np.array(vals, dtype=object).reshape(tuple(reversed(dims)), order="F")
        a = np.frombuffer(raw[:n * dt.size], dtype=dt.numpy()).astype(dt.numpy().newbyteorder("="))
        if dt.kind == "b" and dt.size == 1:
            a = a.astype(bool)
        if not dims:
            return a[0].item()
        return a.reshape(tuple(reversed(dims)), order="F")

    def _global_heap_object(self, addr, index):
        h = self.read_at(addr, 16)
        if h[:4] != b"GCOL":
            raise HDF5Error("bad global heap collection")
        size = struct.unpack_from("<Q", h, 8)[0]
        data = self.read_at(addr, size)
        p = 16
        while p + 16 <= size:
            idx, _ref = struct.unpack_from("<HH", data, p)
            osize = struct.unpack_from("<Q", data, p + 8)[0]
            if idx == index:
                return data[p + 16:p + 16 + osize]
            if idx == 0:
                break
            p += 16 + osize + ((-osize) % 8)
        raise HDF5Error("global heap object not found")

    def close(self):
        self.f.close()


# ---------------------------------------------------------------------------
# the in-memory tree and the file object
# ---------------------------------------------------------------------------
class _Group(dict):
    """name -> _Group | ('addr', object header address) | ('new', value).  ``addr`` and ``stab``
    (B-tree and heap addresses) locate the group on disk; ``dirty`` marks a changed group."""

    def __init__(self):
        super().__init__()
        self.addr = None
        self.stab = None
        self.dirty = True


def _split(path: str):
    parts = [p for p in path.split("/") if p]
    if not parts:
        raise HDF5Error("empty path")
    return parts


class File:
    """An HDF5 file opened like HDF5.jl's ``h5open(path, mode)``: "r" reads, "w" truncates,
    "cw" creates or appends."""

    def __init__(self, path, mode: str = "r"):
        self.path = os.fspath(path)
        self.mode = mode
        self.root = _Group()
        self._r = None
        self._dirty = False
        if mode == "w" or (mode == "cw" and not os.path.exists(self.path)):
            self._new = True
            self._dirty = True
        elif mode in ("r", "cw", "r+"):
            self._new = False
            self._r = _Reader(self.path)
            self._load(self._r.root[1], self.root)
        else:
            raise HDF5Error("unknown mode " + mode)

    # -- reading the existing tree
    def _load(self, ohdr, group):
        links = self._r.group_links(ohdr)
        if links is None:
            raise HDF5Error("object at %d is not a group" % ohdr)
        group.addr, group.stab, group.dirty = ohdr, self._r.last_stab, False
        for name, addr in links.items():
            msgs = self._r.messages(addr)
            if any(t == MSG_STAB for t, _ in msgs):
                g = _Group()
                group[name] = g
                self._load(addr, g)
            else:
                group[name] = ("addr", addr)

    def _node(self, path):
        node = self.root
        for p in _split(path):
            if not isinstance(node, _Group) or p not in node:
                raise KeyError(path)
            node = node[p]
        return node

    def __contains__(self, path):
        try:
            self._node(path)
            return True
        except KeyError:
            return False

    haskey = __contains__

    def keys(self, path: str = "/"):
        node = self.root if path in ("", "/") else self._node(path)
        if not isinstance(node, _Group):
            raise HDF5Error(path + " is not a group")
        return sorted(node.keys(), key=lambda s: s.encode("utf-8"))

    def __getitem__(self, path):
        return self.read(path)

    def read(self, path):
        node = self._node(path)
        if isinstance(node, _Group):
            raise HDF5Error(path + " is a group")
        kind, val = node
        if kind == "addr":
            return self._r.dataset(val)
        return _normalise(val)

    # -- writing
    def __setitem__(self, path, value):
        if self.mode == "r":
            raise HDF5Error("file opened read-only")
        parts = _split(path)
        node = self.root
        chain = [node]
        for p in parts[:-1]:
            nxt = node.get(p)
            if nxt is None:
                nxt = node[p] = _Group()
            elif not isinstance(nxt, _Group):
                raise HDF5Error("%s: %s is a dataset" % (path, p))
            node = nxt
            chain.append(node)
        if parts[-1] in node:
            raise HDF5Error("%s exists already" % path)
        node[parts[-1]] = ("new", _normalise(value))
        for g in chain:
            g.dirty = True
        self._dirty = True

    def close(self):
        if self._dirty and self.mode != "r":
            self._flush()
        if self._r:
            self._r.close()
            self._r = None
        self._dirty = False

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _flush(self):
        """Append the new datasets and every group's metadata, then point the superblock at the
        new root (written last: an interrupted flush leaves the previous state readable)."""
        if self._new:
            fh = open(self.path, "w+b")
            fh.write(b"\0" * 96)
            base_off, sb_pos = 0, 0
        else:
            base_off, sb_pos = self._r.base_addr, self._r.sb_offset
            self._r.close()
            self._r = None
            fh = open(self.path, "r+b")
        fh.seek(0, os.SEEK_END)
        end = fh.tell()
        buf = bytearray()

        def append(b: bytes) -> int:
            nonlocal end
            pad = (-end) % 8
            buf.extend(b"\0" * pad)
            end += pad
            addr = end - base_off
            buf.extend(b)
            end += len(b)
            if len(buf) > (64 << 20):
                fh.write(bytes(buf))
                buf.clear()
            return addr

        def write_dataset(v) -> int:
            if isinstance(v, str):
                data = v.encode("utf-8")
                size = max(len(data), 1)
                dt = _datatype_message("s", size)
                ds = _dataspace_message([])
                raw = data + b"\0" * (size - len(data))
            else:
                a = np.asarray(v)
                if a.dtype == bool:
                    dt, raw = _datatype_message("b1"), np.asfortranarray(a).astype(np.uint8).tobytes(order="F")
                elif a.dtype.kind in "iu":
                    dt, raw = _datatype_message("i8"), np.asfortranarray(a).astype("<i8").tobytes(order="F")
                elif a.dtype.kind == "f":
                    dt, raw = _datatype_message("f8"), np.asfortranarray(a).astype("<f8").tobytes(order="F")
                else:
                    raise HDF5Error("unsupported value type %s" % a.dtype)
                ds = _dataspace_message(list(reversed(a.shape)))
            daddr = append(raw) if raw else UNDEF
            layout = struct.pack("<BBQQ", 3, 1, daddr, len(raw))
            return append(_object_header([(MSG_DATASPACE, ds), (MSG_DATATYPE, dt), (MSG_LAYOUT, layout)]))

        def write_btree(children, level):
            """B-tree nodes over (child address, largest name offset) pairs; returns the root."""
            per = 2 * INTERNAL_K
            nodes = []
            for s in range(0, len(children), per):
                part = children[s:s + per]
                node = b"TREE" + bytes([0, level]) + struct.pack("<HQQ", len(part), UNDEF, UNDEF)
                left = 0 if s == 0 else children[s - 1][1]
                for i, (addr, _) in enumerate(part):
                    node += struct.pack("<QQ", left if i == 0 else part[i - 1][1], addr)
                node += struct.pack("<Q", part[-1][1])
                node += b"\0" * 16 * (per - len(part))
                nodes.append((append(node), part[-1][1]))
            return nodes[0][0] if len(nodes) == 1 else write_btree(nodes, level + 1)

        def write_group(g: _Group) -> tuple:
            if not g.dirty and g.addr is not None:
                return g.addr, g.stab[0], g.stab[1]
            entries = []
            for name in sorted(g.keys(), key=lambda s: s.encode("utf-8")):
                node = g[name]
                if isinstance(node, _Group):
                    oh, bt, hp = write_group(node)
                    entries.append((name, oh, 1, (bt, hp)))
                elif node[0] == "addr":
                    entries.append((name, node[1], 0, (0, 0)))
                else:
                    entries.append((name, write_dataset(node[1]), 0, (0, 0)))
                    g[name] = ("addr", entries[-1][1])
            # local heap: "" at offset 0, the names (each null terminated, 8-byte padded), then one
            # free block (next = 1, the end of the free list, and its size) as libhdf5 lays it out
            heap = bytearray(b"\0" * 8)
            offs = []
            for name, *_ in entries:
                offs.append(len(heap))
                heap.extend(_pad8(name.encode("utf-8") + b"\0"))
            free_off = len(heap)
            heap.extend(struct.pack("<QQ", 1, 16))
            haddr_data = append(bytes(heap))
            hdr = b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap), free_off, haddr_data)
            haddr = append(hdr)
            # symbol table nodes of 2 LEAF_K links, under a B-tree keyed by their largest name
            per = 2 * LEAF_K
            leaves = []
            for s in range(0, max(len(entries), 1), per):
                ch = list(range(s, min(s + per, len(entries))))
                body = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(ch))
                for k in ch:
                    name, oh, cache, (bt, hp) = entries[k]
                    body += struct.pack("<QQI4xQQ", offs[k], oh, cache, bt, hp)
                body += b"\0" * (40 * (per - len(ch)))
                leaves.append((append(body), offs[ch[-1]] if ch else 0))
            baddr = write_btree(leaves, 0)
            oh = append(_object_header([(MSG_STAB, struct.pack("<QQ", baddr, haddr))]))
            g.addr, g.stab, g.dirty = oh, (baddr, haddr), False
            return oh, baddr, haddr

        root_oh, root_bt, root_hp = write_group(self.root)
        # superblock (version 0), written in place
        sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", LEAF_K, INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", base_off, UNDEF, end - base_off, UNDEF)
        sb += struct.pack("<QQI4xQQ", 0, root_oh, 1, root_bt, root_hp)
        # every group node of the file is now one written with these K values; libhdf5's old
        # nodes of an appended file are no longer referenced
        fh.write(bytes(buf))
        fh.flush()
        fh.seek(sb_pos)
        fh.write(sb)
        fh.close()
        self._new = False
        self._r = _Reader(self.path)
        self.root = _Group()
        self._load(self._r.root[1], self.root)


def _normalise(v):
    if isinstance(v, (str, np.ndarray)):
        return v
    if isinstance(v, (bool, np.bool_)):
        return bool(v)
    if isinstance(v, (int, np.integer)):
        return int(v)
    if isinstance(v, (float, np.floating)):
        return float(v)
    return np.asarray(v)


def h5open(path, mode: str = "r") -> File:
    return File(path, mode)
