"""A small HDF5 reader and writer for the files CATO reads and writes, with no HDF5 library.

The reference's initial conditions come from pycato through h5py
(``pycato/generate_initial_grids.py:603-672``: root-level datasets, gzip-compressed chunks, a
``units`` string attribute each) and its contours go out through the HDF5 library
(``contour_writer.f90:193-384``).  Neither machine of this build has h5py or libhdf5, so this
module implements the part of the format those files use, from The HDF Group's public "HDF5 File
Format Specification" (version 3.0):

* superblock versions 0 and 1 (8-byte addresses and lengths);
* version-1 object headers with continuation blocks;
* groups stored as symbol tables (version-1 B-trees of type 0, symbol-table nodes, local heap);
* the dataspace, datatype (fixed-point, IEEE floating point, fixed- and variable-length strings),
  fill value, data layout (compact, contiguous, chunked), filter pipeline (deflate, shuffle,
  Fletcher-32) and attribute messages;
* chunk indexes as version-1 B-trees of type 1, and variable-length data in global heaps.

Reading returns each dataset as numpy stores it in the file (C order of the file's dimensions).
Writing produces the same structures (superblock version 0, one symbol-table root group,
contiguous datasets, fixed-length string attributes), the format every HDF5 library version
reads.  Newer structures (version-2 object headers, link messages, fractal heaps, version-2
B-trees) raise :class:`H5Error`.
"""
from __future__ import annotations

import mmap
import struct
import zlib

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(ValueError):
    """A file this module cannot read (not HDF5, or a structure outside the subset)."""


def _pad8(n: int) -> int:
    return (n + 7) & ~7


# ---------------------------------------------------------------------------------------------
# reading
# ---------------------------------------------------------------------------------------------
class _Type:
    """A decoded datatype message: numpy dtype, or a string kind."""

    def __init__(self, kind: str, dtype=None, size: int = 0, base=None):
        self.kind = kind      # "num", "str" (fixed length), "vlen_str"
        self.dtype = dtype
        self.size = size
        self.base = base


class _Object:
    def __init__(self):
        self.shape = None     # () for a scalar
        self.type = None
        self.layout = None
        self.filters = []
        self.attrs = {}
        self.symtab = None    # (btree, heap) of a group


class H5File:
    """``H5File(path)``: ``keys()`` of the root group, ``read(name)`` a dataset,
    ``attrs(name)`` its attributes (``""`` is the root group)."""

    def __init__(self, path: str):
        self._f = open(path, "rb")
        try:
            self._m = mmap.mmap(self._f.fileno(), 0, access=mmap.ACCESS_READ)
        except ValueError as exc:
            self._f.close()
            raise H5Error(f"{path}: empty file") from exc
        m = self._m
        if m[:8] != _SIG:
            self.close()
            raise H5Error(f"{path}: not an HDF5 file (superblock signature)")
        ver = m[8]
        if ver not in (0, 1):
            self.close()
            raise H5Error(f"{path}: superblock version {ver} (only 0 and 1)")
        if m[13] != 8 or m[14] != 8:
            self.close()
            raise H5Error(f"{path}: addresses of {m[13]} and lengths of {m[14]} bytes")
        pos = 24 + (4 if ver == 1 else 0)
        self._base = struct.unpack_from("<Q", m, pos)[0]
        root = pos + 32  # base, free-space, end-of-file and driver addresses
        self._root = struct.unpack_from("<Q", m, root + 8)[0]
        self._objs = {}

    def close(self):
        if getattr(self, "_m", None) is not None:
            self._m.close()
            self._m = None
        if getattr(self, "_f", None) is not None:
            self._f.close()
            self._f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- low level -----------------------------------------------------------------------------
    def _u(self, fmt: str, pos: int):
        return struct.unpack_from("<" + fmt, self._m, self._base + pos)

    def _bytes(self, pos: int, n: int) -> bytes:
        a = self._base + pos
        return self._m[a:a + n]

    def _messages(self, addr: int):
        """(type, data) of every message of the version-1 object header at addr."""
        if self._bytes(addr, 4) == b"OHDR":
            raise H5Error("version-2 object headers are not supported")
        ver, nmsg, _refs, size = (self._bytes(addr, 1)[0],) + self._u("HIL", addr + 2)
        if ver != 1:
            raise H5Error(f"object header version {ver}")
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            p, end = start, start + length
            while p + 8 <= end and len(out) < nmsg:
                mtype, msize = self._u("HH", p)
                data = self._bytes(p + 8, msize)
                if mtype == 0x10:  # continuation
                    off, ln = struct.unpack_from("<QQ", data, 0)
                    blocks.append((off, ln))
                out.append((mtype, data))
                p += 8 + msize
        return out

    def _heap_name(self, heap: int, off: int) -> str:
        if self._bytes(heap, 4) != b"HEAP":
            raise H5Error("local heap signature")
        seg = self._u("Q", heap + 24)[0]
        b = self._bytes(seg + off, 4096)
        return b[:b.index(b"\0")].decode()

    def _btree_children(self, addr: int, ntype: int, rank1: int = 0):
        """Leaf entries of a version-1 B-tree: (key bytes, child address)."""
        if self._bytes(addr, 4) != b"TREE":
            raise H5Error("B-tree signature")
        t, level = self._bytes(addr + 4, 2)
        if t != ntype:
            raise H5Error(f"B-tree node type {t}, expected {ntype}")
        used = self._u("H", addr + 6)[0]
        ksize = 8 if ntype == 0 else 8 + 8 * rank1
        p = addr + 24
        out = []
        for _ in range(used):
            key = self._bytes(p, ksize)
            child = self._u("Q", p + ksize)[0]
            p += ksize + 8
            if level > 0:
                out.extend(self._btree_children(child, ntype, rank1))
            else:
                out.append((key, child))
        return out

    def _group_entries(self, btree: int, heap: int) -> dict:
        out = {}
        for _key, snod in self._btree_children(btree, 0):
            if self._bytes(snod, 4) != b"SNOD":
                raise H5Error("symbol table node signature")
            n = self._u("H", snod + 6)[0]
            for i in range(n):
                e = snod + 8 + 40 * i
                name_off, ohdr = self._u("QQ", e)
                out[self._heap_name(heap, name_off)] = ohdr
        return out

    def _type(self, d: bytes, pos: int = 0) -> tuple[_Type, int]:
        """Decode a datatype message at d[pos:]; returns the type and its encoded length."""
        cls, bf0 = d[pos] & 0x0F, d[pos + 1]
        size = struct.unpack_from("<I", d, pos + 4)[0]
        order = ">" if bf0 & 1 else "<"
        if cls == 0:
            signed = (bf0 >> 3) & 1
            return _Type("num", np.dtype(f"{order}{'i' if signed else 'u'}{size}")), 12
        if cls == 1:
            if size not in (2, 4, 8):
                raise H5Error(f"floating point of {size} bytes")
            return _Type("num", np.dtype(f"{order}f{size}")), 20
        if cls == 3:
            return _Type("str", size=size), 8
        if cls == 9 and (bf0 & 0x0F) == 1:
            base, blen = self._type(d, pos + 8)
            return _Type("vlen_str", size=size, base=base), 8 + blen
        raise H5Error(f"datatype class {cls}")

    @staticmethod
    def _space(d: bytes) -> tuple:
        ver, rank, flags = d[0], d[1], d[2]
        if ver == 1:
            p = 8
        elif ver == 2:
            if d[3] == 2:  # null dataspace
                return None
            p = 4
        else:
            raise H5Error(f"dataspace version {ver}")
        return tuple(struct.unpack_from(f"<{rank}Q", d, p)) if rank else ()

    def _object(self, addr: int) -> _Object:
        if addr in self._objs:
            return self._objs[addr]
        o = _Object()
        for mtype, d in self._messages(addr):
            if mtype == 0x0001:
                o.shape = self._space(d)
            elif mtype == 0x0003:
                o.type = self._type(d)[0]
            elif mtype == 0x0008:
                o.layout = self._layout(d)
            elif mtype == 0x000B:
                o.filters = self._filters(d)
            elif mtype == 0x000C:
                name, value = self._attribute(d)
                o.attrs[name] = value
            elif mtype == 0x0011:
                o.symtab = struct.unpack_from("<QQ", d, 0)
        self._objs[addr] = o
        return o

    @staticmethod
    def _layout(d: bytes):
        ver = d[0]
        if ver != 3:
            raise H5Error(f"data layout version {ver} (only 3)")
        cls = d[1]
        if cls == 0:
            n = struct.unpack_from("<H", d, 2)[0]
            return ("compact", bytes(d[4:4 + n]))
        if cls == 1:
            return ("contiguous",) + struct.unpack_from("<QQ", d, 2)
        if cls == 2:
            rank1 = d[2]
            btree = struct.unpack_from("<Q", d, 3)[0]
            dims = struct.unpack_from(f"<{rank1}I", d, 11)
            return ("chunked", btree, dims)
        raise H5Error(f"data layout class {cls}")

    @staticmethod
    def _filters(d: bytes) -> list:
        ver, n = d[0], d[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = struct.unpack_from("<H", d, p)[0]
            if ver == 1 or fid >= 256:
                nlen, _flags, nval = struct.unpack_from("<HHH", d, p + 2)
                p += 8
            else:
                nlen = 0
                _flags, nval = struct.unpack_from("<HH", d, p + 2)
                p += 6
            p += _pad8(nlen) if ver == 1 else nlen
            vals = struct.unpack_from(f"<{nval}I", d, p)
            p += 4 * nval + (4 if ver == 1 and nval % 2 else 0)
            out.append((fid, vals))
        return out

    def _attribute(self, d: bytes):
        ver = d[0]
        nsz, tsz, ssz = struct.unpack_from("<HHH", d, 2)
        if ver == 1:
            p = 8
            name = bytes(d[p:p + nsz]).rstrip(b"\0").decode()
            p += _pad8(nsz)
            typ = self._type(d, p)[0]
            p += _pad8(tsz)
            shape = self._space(d[p:p + ssz])
            p += _pad8(ssz)
        elif ver in (2, 3):
            p = 8 + (1 if ver == 3 else 0)
            name = bytes(d[p:p + nsz]).rstrip(b"\0").decode()
            p += nsz
            typ = self._type(d, p)[0]
            p += tsz
            shape = self._space(d[p:p + ssz])
            p += ssz
        else:
            raise H5Error(f"attribute message version {ver}")
        n = int(np.prod(shape)) if shape else 1
        return name, self._values(typ, bytes(d[p:]), n, shape)

    def _gheap_object(self, coll: int, index: int) -> bytes:
        if self._bytes(coll, 4) != b"GCOL":
            raise H5Error("global heap signature")
        size = self._u("Q", coll + 8)[0]
        p, end = coll + 16, coll + size
        while p + 16 <= end:
            idx, _ref, _res, osz = self._u("HHIQ", p)
            if idx == 0:
                break
            if idx == index:
                return self._bytes(p + 16, osz)
            p += 16 + _pad8(osz)
        raise H5Error(f"global heap object {index} not found")

    def _values(self, typ: _Type, raw: bytes, n: int, shape):
        if typ.kind == "num":
            a = np.frombuffer(raw, dtype=typ.dtype, count=n).astype(typ.dtype.newbyteorder("="))
            return a.reshape(shape) if shape else a[0]
        if typ.kind == "str":
            vals = [raw[i * typ.size:(i + 1) * typ.size].split(b"\0")[0].decode().rstrip()
                    for i in range(n)]
        else:  # variable length: length, global heap collection, object index
            vals = []
            for i in range(n):
                _ln, coll, idx = struct.unpack_from("<IQI", raw, 16 * i)
                vals.append(self._gheap_object(coll, idx).decode())
        return vals[0] if not shape else np.array(vals, dtype=object).reshape(shape)

    # -- public --------------------------------------------------------------------------------
    def _lookup(self, name: str) -> _Object:
        addr = self._root
        for part in [p for p in name.strip("/").split("/") if p]:
            g = self._object(addr)
            if g.symtab is None:
                raise H5Error(f"{name}: not a group on the way")
            entries = self._group_entries(*g.symtab)
            if part not in entries:
                raise KeyError(name)
            addr = entries[part]
        return self._object(addr)

    def keys(self, group: str = "") -> list:
        g = self._lookup(group)
        if g.symtab is None:
            raise H5Error(f"{group!r} is not a group")
        return sorted(self._group_entries(*g.symtab))

    def attrs(self, name: str = "") -> dict:
        return dict(self._lookup(name).attrs)

    def read(self, name: str):
        o = self._lookup(name)
        if o.layout is None or o.type is None:
            raise H5Error(f"{name} is not a dataset")
        shape = o.shape or ()
        n = int(np.prod(shape)) if shape else 1
        kind = o.layout[0]
        if kind == "compact":
            return self._values(o.type, o.layout[1], n, shape)
        if kind == "contiguous":
            addr, size = o.layout[1], o.layout[2]
            # an unallocated dataset (never written) reads as zeros
            raw = bytes(size) if addr == _UNDEF else self._bytes(addr, size)
            return self._values(o.type, raw, n, shape)
        if o.type.kind != "num":
            raise H5Error("chunked strings are not supported")
        btree, cdims = o.layout[1], o.layout[2]
        dt = o.type.dtype
        out = np.zeros(shape, dtype=dt.newbyteorder("="))
        rank = len(shape)
        chunk_shape = tuple(cdims[:rank])
        if btree == _UNDEF:
            return out
        for key, addr in self._btree_children(btree, 1, rank + 1):
            csize, mask = struct.unpack_from("<II", key, 0)
            offs = struct.unpack_from(f"<{rank + 1}Q", key, 8)[:rank]
            raw = self._bytes(addr, csize)
            for k, (fid, vals) in reversed(list(enumerate(o.filters))):
                if mask & (1 << k):
                    continue
                if fid == 1:      # deflate
                    raw = zlib.decompress(raw)
                elif fid == 2:    # shuffle: the bytes of each element were grouped by position
                    esz = vals[0] if vals else dt.itemsize
                    b = np.frombuffer(raw, dtype=np.uint8)
                    m = len(b) // esz
                    raw = b[:m * esz].reshape(esz, m).T.tobytes() + b[m * esz:].tobytes()
                elif fid == 3:    # Fletcher-32: a checksum after the data
                    raw = raw[:-4]
                else:
                    raise H5Error(f"filter {fid}")
            block = np.frombuffer(raw, dtype=dt, count=int(np.prod(chunk_shape)))
            block = block.reshape(chunk_shape)
            sel = tuple(slice(o_, min(o_ + c, s)) for o_, c, s in zip(offs, chunk_shape, shape))
            out[sel] = block[tuple(slice(0, s.stop - s.start) for s in sel)]
        return out


def read_dataset(path: str, name: str):
    with H5File(path) as f:
        return f.read(name)


# ---------------------------------------------------------------------------------------------
# writing
# ---------------------------------------------------------------------------------------------
def _dtype_msg(dt: np.dtype) -> bytes:
    dt = np.dtype(dt)
    if dt.kind == "f":
        size = dt.itemsize
        if size == 8:
            sign, eloc, esz, msz, bias = 63, 52, 11, 52, 1023
        elif size == 4:
            sign, eloc, esz, msz, bias = 31, 23, 8, 23, 127
        else:
            raise H5Error(f"float of {size} bytes")
        # class 1 version 1; little endian, mantissa normalisation "implied msb" (2)
        head = bytes([0x11, 0x20, sign, 0]) + struct.pack("<I", size)
        return head + struct.pack("<HHBBBBI", 0, 8 * size, eloc, esz, 0, msz, bias)
    if dt.kind in "iu":
        size = dt.itemsize
        head = bytes([0x10, 0x08 if dt.kind == "i" else 0, 0, 0]) + struct.pack("<I", size)
        return head + struct.pack("<HH", 0, 8 * size)
    raise H5Error(f"dtype {dt}")


def _str_type_msg(n: int) -> bytes:
    # class 3 version 1: fixed length, null terminated, ASCII
    return bytes([0x13, 0x00, 0, 0]) + struct.pack("<I", n)


def _space_msg(shape: tuple) -> bytes:
    return bytes([1, len(shape), 0, 0, 0, 0, 0, 0]) + b"".join(struct.pack("<Q", d) for d in shape)


def _msg(mtype: int, data: bytes, flags: int = 0) -> bytes:
    data = data + bytes(_pad8(len(data)) - len(data))
    return struct.pack("<HHB3x", mtype, len(data), flags) + data


def _attr_msg(name: str, value) -> bytes:
    nm = name.encode() + b"\0"
    if isinstance(value, str):
        raw = value.encode()
        typ = _str_type_msg(len(raw) + 1)
        data = raw + b"\0"
        space = _space_msg(())
    else:
        a = np.asarray(value)
        if a.dtype.kind not in "fiu":
            raise H5Error(f"attribute {name}: {a.dtype}")
        a = a.astype(a.dtype.newbyteorder("<"))
        typ, data, space = _dtype_msg(a.dtype), a.tobytes(), _space_msg(a.shape)
    body = struct.pack("<BBHHH", 1, 0, len(nm), len(typ), len(space))
    body += nm + bytes(_pad8(len(nm)) - len(nm))
    body += typ + bytes(_pad8(len(typ)) - len(typ))
    body += space + bytes(_pad8(len(space)) - len(space))
    return _msg(0x000C, body + data)


def _ohdr(messages: list) -> bytes:
    body = b"".join(messages)
    return struct.pack("<BBHII", 1, 0, len(messages), 1, len(body)) + bytes(4) + body


def write_file(path: str, datasets: dict, root_attrs: dict | None = None) -> None:
    """Write root-level datasets: ``datasets[name] = (array, {attribute: value})``.  Arrays go
    out in their C order (callers that follow h5py's convention pass the transpose of a Fortran
    (i, j) array); a str value is a scalar fixed-length ASCII string dataset, and str attribute
    values are fixed-length ASCII strings."""
    items = {n.strip("/"): v for n, v in datasets.items()}
    if any("/" in n for n in items):
        raise H5Error("root-level datasets only")
    names = sorted(items)  # a symbol-table node lists its entries in name order
    leaf_k = max(4, (len(names) + 1) // 2)
    int_k = 16
    # local heap: the empty name at 0, then the names
    heap_data = bytearray(8)
    name_off = {}
    for n in names:
        name_off[n] = len(heap_data)
        b = n.encode() + b"\0"
        heap_data += b + bytes(_pad8(len(b)) - len(b))
    heap_data += bytes(_pad8(len(heap_data)) - len(heap_data))
    # layout of the file
    sb_size = 96
    pos = sb_size
    root_oh = _ohdr([_msg(0x0011, bytes(16))] +
                    [_attr_msg(k, v) for k, v in (root_attrs or {}).items()])
    root_addr, pos = pos, pos + len(root_oh)
    heap_addr, pos = pos, pos + 32
    heap_seg, pos = pos, pos + len(heap_data)
    tree_size = 24 + (2 * int_k + 1) * 8 + 2 * int_k * 8
    tree_addr, pos = pos, pos + tree_size
    snod_size = 8 + 2 * leaf_k * 40
    snod_addr, pos = pos, pos + snod_size
    # dataset headers, then their data
    headers, arrays = {}, {}
    for n in names:
        arr, attrs = items[n]
        if isinstance(arr, str):
            raw = arr.encode() + b"\0"
            a = np.frombuffer(raw, dtype=f"S{len(raw)}").reshape(())
        else:
            a = np.array(arr, order="C")  # keeps a scalar 0-dimensional
            a = a.astype(a.dtype.newbyteorder("<"))
        arrays[n] = a
        attr_msgs = [_attr_msg(k, v) for k, v in (attrs or {}).items()]
        # placeholder layout; the address is filled in below
        headers[n] = (a, attr_msgs)
    oh_addr = {}
    oh_len = {}
    for n in names:
        a, attr_msgs = headers[n]
        probe = _ohdr(_dataset_msgs(a, 0) + attr_msgs)
        oh_addr[n], oh_len[n] = pos, len(probe)
        pos += len(probe)
    data_addr = {}
    for n in names:
        pos = _pad8(pos)
        data_addr[n] = pos
        pos += arrays[n].nbytes
    eof = _pad8(pos)
    out = bytearray(eof)
    # superblock version 0 and the root symbol-table entry
    sb = _SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", leaf_k, int_k, 0)
    sb += struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
    sb += struct.pack("<QQII", 0, root_addr, 1, 0) + struct.pack("<QQ", tree_addr, heap_addr)
    out[0:len(sb)] = sb
    root_oh = _ohdr([_msg(0x0011, struct.pack("<QQ", tree_addr, heap_addr))] +
                    [_attr_msg(k, v) for k, v in (root_attrs or {}).items()])
    out[root_addr:root_addr + len(root_oh)] = root_oh
    out[heap_addr:heap_addr + 32] = (b"HEAP" + bytes([0, 0, 0, 0]) +
                                     struct.pack("<QQQ", len(heap_data), _UNDEF, heap_seg))
    out[heap_seg:heap_seg + len(heap_data)] = heap_data
    # B-tree (type 0, one leaf): key 0 = the empty name, key 1 = the last name of the node
    tree = b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", 1, _UNDEF, _UNDEF)
    tree += struct.pack("<QQQ", 0, snod_addr, name_off[names[-1]] if names else 0)
    out[tree_addr:tree_addr + len(tree)] = tree
    snod = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(names))
    for n in names:
        snod += struct.pack("<QQII", name_off[n], oh_addr[n], 0, 0) + bytes(16)
    out[snod_addr:snod_addr + len(snod)] = snod
    for n in names:
        a, attr_msgs = headers[n]
        oh = _ohdr(_dataset_msgs(a, data_addr[n]) + attr_msgs)
        assert len(oh) == oh_len[n]
        out[oh_addr[n]:oh_addr[n] + len(oh)] = oh
        out[data_addr[n]:data_addr[n] + a.nbytes] = a.tobytes()
    with open(path, "wb") as fh:
        fh.write(out)


def _dataset_msgs(a: np.ndarray, addr: int) -> list:
    # fill value message version 2: late allocation, write if set, no fill value defined
    typ = _str_type_msg(a.dtype.itemsize) if a.dtype.kind == "S" else _dtype_msg(a.dtype)
    return [_msg(0x0001, _space_msg(a.shape)), _msg(0x0003, typ, 1),
            _msg(0x0005, bytes([2, 2, 2, 0]), 1),
            _msg(0x0008, bytes([3, 1]) + struct.pack("<QQ", addr, a.nbytes))]
