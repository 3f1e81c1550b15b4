"""Minimal HDF5 reader and writer for the archives of the TDSE -> far-field path (no libhdf5).

The pipeline's archives are plain HDF5: groups and contiguous or chunked numeric datasets with
string ``units`` attributes (the merged TDSE outputs, ``1DTDSE/python/merge.py:71-108``; the
far-field results, ``Hankel/Hankel_long_medium_parallel_cluster.py:323-367``; the TDSE library's
own ``save_to_hdf5``, ``1DTDSE/PythonCTDSE/structures.py:301-340, 454-505``; the fields the MPI
driver reads, ``1DTDSE/sources/MPI-TDSE.c:185-190`` with the names of ``h5namelist.h:11-25``).
h5py and libhdf5 are not available here, so this module implements the part of the HDF5 file
format that these files use:

reading
    superblocks 0-3; version 1 object headers and version 2 ("OHDR"/"OCHK") headers with
    continuation blocks; groups as symbol tables (B-tree v1 group nodes, local heaps, symbol
    nodes) or compact link messages; dataspaces (scalar, simple); datatypes fixed-point,
    floating-point, fixed-length string and compound of those; layouts compact, contiguous and
    chunked (B-tree v1 chunk index) with the deflate and shuffle filters; attributes.
writing (mode "w", or "a" which first reads an existing file's tree; written on close)
    superblock 0, groups as symbol tables, datasets of fixed-point, floating-point and
    fixed-length string types -- contiguous, or chunked (B-tree v1 chunk index) with optional
    deflate and shuffle filters (h5py's ``chunks=``, ``compression="gzip"``, ``shuffle=``) --
    scalar and simple dataspaces, attributes of the same types.

Dense (fractal-heap) groups, variable-length types and the version 4 layouts raise
``NotImplementedError`` when they are reached.  The writer lays its files out with the
structures libhdf5 writes for a new file at its default ("earliest") format version: the same
superblock, node sizes (group leaf K 4, internal K 16), local-heap free block and sorted symbol
nodes as the reference's own ``1DTDSE/ionization.h5``.  Reading them back through this reader is
tested; reading them with libhdf5 cannot be tested here.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


class H5FormatError(ValueError):
    pass


# ---------------------------------------------------------------------------------------------
# reading
# ---------------------------------------------------------------------------------------------

def _le(b, off, n):
    return int.from_bytes(b[off:off + n], "little")


def _pad8(n):
    return (n + 7) & ~7


class _Buf:
    """The file's bytes with its sizes of offsets (so) and lengths (sl)."""

    def __init__(self, data: bytes, so: int = 8, sl: int = 8):
        self.d = data
        self.so, self.sl = so, sl

    def u(self, off, n):
        return _le(self.d, off, n)

    def addr(self, off):
        return _le(self.d, off, self.so)

    def length(self, off):
        return _le(self.d, off, self.sl)


def _parse_datatype(b: bytes, off: int = 0):
    """Datatype message -> (numpy dtype, bytes consumed)."""
    cv = b[off]
    cls, ver = cv & 0x0F, cv >> 4
    bits = _le(b, off + 1, 3)
    size = _le(b, off + 4, 4)
    p = off + 8
    order = ">" if bits & 1 else "<"
    if cls == 0:  # fixed-point
        signed = bool(bits & 0x08)
        if size not in (1, 2, 4, 8):
            raise NotImplementedError("fixed-point of %d bytes" % size)
        return np.dtype("%s%s%d" % (order, "i" if signed else "u", size)), p + 4 - off
    if cls == 1:  # floating-point
        if size not in (2, 4, 8):
            raise NotImplementedError("floating-point of %d bytes" % size)
        return np.dtype("%sf%d" % (order, size)), p + 12 - off
    if cls == 3:  # fixed-length string
        return np.dtype("S%d" % size), p - off
    if cls == 6:  # compound
        nm = bits & 0xFFFF
        names, formats, offsets = [], [], []
        for _ in range(nm):
            end = b.index(b"\0", p)
            name = b[p:end].decode()
            p = p + _pad8(end - p + 1) if ver < 3 else end + 1
            if ver == 1:
                moff = _le(b, p, 4)
                p += 4 + 1 + 3 + 4 + 4 + 16  # offset, dimensionality, reserved, permutation, reserved, dims
            elif ver == 2:
                moff = _le(b, p, 4)
                p += 4
            else:
                nb = 1 if size < 256 else 2 if size < 65536 else 3 if size < (1 << 24) else 4
                moff = _le(b, p, nb)
                p += nb
            mdt, used = _parse_datatype(b, p)
            p += used
            names.append(name)
            formats.append(mdt)
            offsets.append(moff)
        return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": size}), p - off
    raise NotImplementedError("HDF5 datatype class %d" % cls)


def _parse_dataspace(b: bytes, sl: int):
    """Dataspace message -> dims tuple (() for a scalar) or None for a null dataspace."""
    ver, rank = b[0], b[1]
    if ver == 1:
        p, kind = 8, (1 if rank > 0 else 0)
    elif ver == 2:
        p, kind = 4, b[3]
    else:
        raise NotImplementedError("dataspace version %d" % ver)
    if kind == 2:
        return None
    return tuple(_le(b, p + i * sl, sl) for i in range(rank))


class _Object:
    """A parsed object header: its messages as (type, data bytes)."""

    def __init__(self, f: "File", addr: int):
        self.f, self.addr = f, addr
        self.msgs = []
        B = f._b
        d = B.d
        if d[addr:addr + 4] == b"OHDR":
            flags = d[addr + 5]
            p = addr + 6
            if flags & 0x20:
                p += 16
            if flags & 0x10:
                p += 4
            nsz = 1 << (flags & 3)
            size0 = B.u(p, nsz)
            p += nsz
            self._read_v2(p, p + size0, flags)
        else:
            if d[addr] != 1:
                raise H5FormatError("object header version %d at %d" % (d[addr], addr))
            nmsg = B.u(addr + 2, 2)
            hsize = B.u(addr + 8, 4)
            self._read_v1(addr + 16, addr + 16 + hsize, nmsg)

    def _read_v1(self, p, end, nmsg):
        B = self.f._b
        blocks = [(p, end)]
        while blocks and len(self.msgs) < nmsg:
            p, end = blocks.pop(0)
            while p + 8 <= end and len(self.msgs) < nmsg:
                mt, ms = B.u(p, 2), B.u(p + 2, 2)
                data = B.d[p + 8:p + 8 + ms]
                p += 8 + ms
                if mt == 0x10:  # continuation: address and length of the next block of messages
                    ca, cl = _le(data, 0, B.so), _le(data, B.so, B.sl)
                    blocks.append((ca, ca + cl))
                self.msgs.append((mt, data))

    def _read_v2(self, p, end, flags):
        B = self.f._b
        blocks = [(p, end)]
        h = 4 + (2 if flags & 0x04 else 0)
        while blocks:
            p, end = blocks.pop(0)
            while p + h <= end:
                mt, ms = B.d[p], B.u(p + 1, 2)
                data = B.d[p + h:p + h + ms]
                p += h + ms
                if mt == 0x10:
                    ca, cl = _le(data, 0, B.so), _le(data, B.so, B.sl)
                    if B.d[ca:ca + 4] != b"OCHK":
                        raise H5FormatError("continuation block without OCHK")
                    blocks.append((ca + 4, ca + cl - 4))
                self.msgs.append((mt, data))
            # what is left of a block (a gap, the checksum) holds no message

    def find(self, mt):
        return [d for t, d in self.msgs if t == mt]


class Attributes:
    def __init__(self, items=None):
        self._d = dict(items or {})

    def __getitem__(self, k):
        return self._d[k]

    def __setitem__(self, k, v):
        self._d[k] = v

    def __contains__(self, k):
        return k in self._d

    def keys(self):
        return self._d.keys()

    def items(self):
        return self._d.items()


def _parse_attribute(f: "File", b: bytes):
    ver = b[0]
    nlen, tlen, slen = _le(b, 2, 2), _le(b, 4, 2), _le(b, 6, 2)
    p = 8 + (1 if ver == 3 else 0)
    pad = _pad8 if ver == 1 else (lambda n: n)
    name = b[p:p + nlen].rstrip(b"\0").decode()
    p += pad(nlen)
    dt, _ = _parse_datatype(b, p)
    p += pad(tlen)
    dims = _parse_dataspace(b[p:p + slen], f._b.sl)
    p += pad(slen)
    if dims is None:
        return name, None
    n = int(np.prod(dims)) if dims else 1
    val = np.frombuffer(b[p:p + n * dt.itemsize], dtype=dt, count=n)
    return name, (val.reshape(dims) if dims else val[0])


class Dataset:
    def __init__(self, f: "File", obj: _Object, name: str):
        self.file, self.name = f, name
        sp, ty, ly = obj.find(0x0001), obj.find(0x0003), obj.find(0x0008)
        if not (sp and ty and ly):
            raise H5FormatError("%s: not a dataset" % name)
        self.shape = _parse_dataspace(sp[0], f._b.sl) or ()
        self.dtype, _ = _parse_datatype(ty[0])
        self._layout = ly[0]
        self._filters = self._parse_filters(obj.find(0x000B))
        self.attrs = Attributes(_parse_attribute(f, a) for a in obj.find(0x000C))

    @staticmethod
    def _parse_filters(msgs):
        if not msgs:
            return []
        b = msgs[0]
        ver, nf = b[0], b[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(nf):
            fid = _le(b, p, 2)
            if ver == 1 or fid >= 256:
                nl = _le(b, p + 2, 2)
                p += 2
            else:
                nl = 0
            nv = _le(b, p + 4, 2)
            p += 6
            p += _pad8(nl) if ver == 1 else nl
            vals = [_le(b, p + 4 * i, 4) for i in range(nv)]
            p += 4 * nv
            if ver == 1 and nv % 2:
                p += 4
            out.append((fid, vals))
        return out

    def _unfilter(self, raw: bytes, mask: int):
        for i, (fid, vals) in reversed(list(enumerate(self._filters))):
            if mask & (1 << i):
                continue
            if fid == 1:  # deflate
                raw = zlib.decompress(raw)
            elif fid == 2:  # shuffle: bytes grouped by position within the element
                es = vals[0] if vals else self.dtype.itemsize
                a = np.frombuffer(raw, dtype=np.uint8)
                n = a.size // es
                raw = a[:n * es].reshape(es, n).T.tobytes() + raw[n * es:]
            else:
                raise NotImplementedError("HDF5 filter %d" % fid)
        return raw

    def _read(self):
        B = self.file._b
        L = self._layout
        ver = L[0]
        n = int(np.prod(self.shape)) if self.shape else 1
        nbytes = n * self.dtype.itemsize
        if ver in (1, 2):
            rank, cls = L[1], L[2]
            p = 8
            if cls == 0:
                p += 4 * rank
                raw = L[p + 4:p + 4 + _le(L, p, 4)]
            elif cls == 1:
                a = _le(L, p, B.so)
                raw = B.d[a:a + nbytes] if a != _UNDEF else b"\0" * nbytes
            else:
                cdims = [_le(L, p + B.so + 4 * i, 4) for i in range(rank)]
                return self._read_chunked(_le(L, p, B.so), cdims)
        elif ver == 3:
            cls = L[1]
            if cls == 0:
                raw = L[4:4 + _le(L, 2, 2)]
            elif cls == 1:
                a = _le(L, 2, B.so)
                raw = B.d[a:a + nbytes] if a != _UNDEF else b"\0" * nbytes
            elif cls == 2:
                rank = L[2]
                cdims = [_le(L, 3 + B.so + 4 * i, 4) for i in range(rank)]
                return self._read_chunked(_le(L, 3, B.so), cdims)
            else:
                raise NotImplementedError("layout class %d" % cls)
        else:
            raise NotImplementedError("data layout version %d" % ver)
        if len(raw) < nbytes:
            raise H5FormatError("%s: data truncated" % self.name)
        arr = np.frombuffer(raw[:nbytes], dtype=self.dtype, count=n)
        return arr.reshape(self.shape) if self.shape else arr[0]

    def _read_chunked(self, btree, cdims):
        """B-tree v1 chunk index (node type 1): each key holds the chunk's stored size, its
        filter mask and its offsets; level-0 children are the chunks."""
        B = self.file._b
        rank = len(self.shape)
        chunk = tuple(cdims[:rank])
        out = np.zeros(self.shape, dtype=self.dtype)
        if btree == _UNDEF:
            return out
        ksize = 8 + 8 * (rank + 1)
        stack = [btree]
        while stack:
            a = stack.pop()
            if B.d[a:a + 4] != b"TREE" or B.d[a + 4] != 1:
                raise H5FormatError("chunk B-tree node expected at %d" % a)
            level, used = B.d[a + 5], B.u(a + 6, 2)
            p = a + 8 + 2 * B.so
            for _ in range(used):
                csize, mask = B.u(p, 4), B.u(p + 4, 4)
                offs = [B.u(p + 8 + 8 * k, 8) for k in range(rank)]
                child = B.addr(p + ksize)
                p += ksize + B.so
                if level > 0:
                    stack.append(child)
                    continue
                raw = self._unfilter(B.d[child:child + csize], mask)
                blk = np.frombuffer(raw, dtype=self.dtype, count=int(np.prod(chunk))).reshape(chunk)
                sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, chunk, self.shape))
                out[sl] = blk[tuple(slice(0, s.stop - s.start) for s in sl)]
        return out

    def __getitem__(self, key):
        a = self._read()
        if key == () or key is Ellipsis:
            return a
        return np.asarray(a)[key]

    def __len__(self):
        return self.shape[0]

    @property
    def ndim(self):
        return len(self.shape)


class Group:
    def __init__(self, f: "File", obj: _Object, name: str):
        self.file, self.name, self._obj = f, name, obj
        self.attrs = Attributes(_parse_attribute(f, a) for a in obj.find(0x000C))
        self._links = None

    def _members(self):
        if self._links is None:
            links = {}
            st = self._obj.find(0x0011)
            if st:
                so = self.file._b.so
                links = self.file._symbol_table(_le(st[0], 0, so), _le(st[0], so, so))
            for lm in self._obj.find(0x0006):
                nm, a = self.file._link_message(lm)
                if a is not None:
                    links[nm] = a
            li = self._obj.find(0x0002)
            if li and not st and not self._obj.find(0x0006):
                b = li[0]
                heap_addr = _le(b, 2 + (8 if b[1] & 1 else 0), self.file._b.so)
                if heap_addr != _UNDEF:
                    raise NotImplementedError("dense (fractal heap) group storage")
            self._links = links
        return self._links

    def keys(self):
        return list(self._members().keys())

    def __iter__(self):
        return iter(self.keys())

    def __contains__(self, path):
        try:
            self[path]
            return True
        except KeyError:
            return False

    def __getitem__(self, path):
        node = self
        for part in [p for p in path.split("/") if p]:
            if not isinstance(node, Group):
                raise KeyError(path)
            m = node._members()
            if part not in m:
                raise KeyError(path)
            node = self.file._open(m[part], node.name.rstrip("/") + "/" + part)
        return node

    def items(self):
        return [(k, self[k]) for k in self.keys()]


class File(Group):
    """``File(path)`` reads an HDF5 file; ``File(path, "w")`` builds a tree written on close."""

    def __new__(cls, path, mode="r"):
        if mode == "r":
            return super().__new__(cls)
        if mode == "w":
            return _Writer(path)
        if mode == "a":
            return _Writer(path, keep=True)
        raise NotImplementedError("mode %r: only 'r', 'w' and 'a'" % mode)

    def __init__(self, path, mode="r"):
        with open(path, "rb") as fh:
            data = fh.read()
        i = 0
        while data[i:i + 8] != _SIG:  # the superblock may follow a user block of 512 * 2^k bytes
            i = 512 if i == 0 else 2 * i
            if i >= len(data):
                raise H5FormatError("%s: not an HDF5 file" % path)
        d = data[i:]
        ver = d[8]
        if ver in (0, 1):
            so, sl = d[13], d[14]
            self._b = _Buf(d, so, sl)
            p = 24 + (4 if ver == 1 else 0) + 4 * so  # base, free space, end of file, driver info
            root = self._b.addr(p + so)  # object header of the root symbol table entry
        elif ver in (2, 3):
            so, sl = d[9], d[10]
            self._b = _Buf(d, so, sl)
            root = self._b.addr(12 + 3 * so)
        else:
            raise NotImplementedError("superblock version %d" % ver)
        self.path = path
        self._cache = {}
        Group.__init__(self, self, _Object(self, root), "/")

    def _open(self, addr, name):
        if addr not in self._cache:
            obj = _Object(self, addr)
            self._cache[addr] = Dataset(self, obj, name) if obj.find(0x0008) else Group(self, obj, name)
        return self._cache[addr]

    def _symbol_table(self, btree, heap):
        B = self._b
        if B.d[heap:heap + 4] != b"HEAP":
            raise H5FormatError("local heap expected at %d" % heap)
        data_addr = B.addr(heap + 8 + 2 * B.sl)

        def name_at(off):
            s = data_addr + off
            return B.d[s:B.d.index(b"\0", s)].decode()

        out = {}
        stack = [btree]
        while stack:
            a = stack.pop()
            if B.d[a:a + 4] != b"TREE" or B.d[a + 4] != 0:
                raise H5FormatError("group B-tree node expected at %d" % a)
            level, used = B.d[a + 5], B.u(a + 6, 2)
            p = a + 8 + 2 * B.so
            for _ in range(used):
                child = B.addr(p + B.sl)
                p += B.sl + B.so
                if level > 0:
                    stack.append(child)
                    continue
                if B.d[child:child + 4] != b"SNOD":
                    raise H5FormatError("symbol node expected at %d" % child)
                q = child + 8
                for _ in range(B.u(child + 6, 2)):
                    out[name_at(B.length(q))] = B.addr(q + B.sl)
                    q += B.sl + B.so + 4 + 4 + 16
        return out

    def _link_message(self, b):
        flags = b[1]
        p = 2
        ltype = 0
        if flags & 0x08:
            ltype = b[p]
            p += 1
        if flags & 0x04:
            p += 8
        if flags & 0x10:
            p += 1
        nb = 1 << (flags & 3)
        nl = _le(b, p, nb)
        p += nb
        name = b[p:p + nl].decode()
        p += nl
        if ltype != 0:  # soft and external links are not followed
            return name, None
        return name, _le(b, p, self._b.so)

    def close(self):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False


# ---------------------------------------------------------------------------------------------
# writing (superblock 0, symbol-table groups, contiguous datasets)
# ---------------------------------------------------------------------------------------------

_LEAF_K, _INTERNAL_K = 4, 16  # symbol nodes of 2*4 entries; group B-tree nodes of 2*16 children


def _dtype_message(dt: np.dtype) -> bytes:
    dt = np.dtype(dt)
    if dt.kind in "iu":
        bits = (0x08 if dt.kind == "i" else 0) | (1 if dt.byteorder == ">" else 0)
        return bytes([0x10, bits, 0, 0]) + struct.pack("<IHH", dt.itemsize, 0, 8 * dt.itemsize)
    if dt.kind == "f":
        # IEEE layout: bit offset, precision, exponent location and size, mantissa location and
        # size, exponent bias; class bits: byte order, implied leading mantissa bit, sign position
        props = {8: (64, 52, 11, 52, 1023), 4: (32, 23, 8, 23, 127), 2: (16, 10, 5, 10, 15)}[dt.itemsize]
        prec, eloc, esz, msz, bias = props
        body = struct.pack("<HHBBBBI", 0, prec, eloc, esz, 0, msz, bias)
        order = 1 if dt.byteorder == ">" else 0
        return bytes([0x11, order | (2 << 4), prec - 1, 0]) + struct.pack("<I", dt.itemsize) + body
    if dt.kind == "S":
        return bytes([0x13, 0, 0, 0]) + struct.pack("<I", dt.itemsize)  # null-terminated ASCII
    raise NotImplementedError("writing dtype %s" % dt)


def _dataspace_message(shape) -> bytes:
    return bytes([1, len(shape), 0, 0]) + b"\0" * 4 + b"".join(struct.pack("<Q", s) for s in shape)


def _message(mt, data, flags=0):
    data = data + b"\0" * (_pad8(len(data)) - len(data))
    return struct.pack("<HHB3x", mt, len(data), flags) + data


def _as_array(v):
    if isinstance(v, str):
        v = v.encode()
    a = np.asarray(v)
    if a.dtype.kind == "U":
        a = np.char.encode(a, "ascii")
    if a.dtype.kind == "b":
        a = a.astype(np.uint8)
    if a.dtype.kind == "c":
        raise NotImplementedError("complex data: store real and imaginary parts in a trailing axis of 2")
    if a.dtype.kind not in "iufS":
        raise NotImplementedError("writing dtype %s" % a.dtype)
    if a.dtype.byteorder == ">":
        a = a.astype(a.dtype.newbyteorder("<"))
    return a


def _attribute_message(name, value) -> bytes:
    a = _as_array(value)
    nm = name.encode() + b"\0"
    dtm, spm = _dtype_message(a.dtype), _dataspace_message(a.shape)
    body = struct.pack("<BBHHH", 1, 0, len(nm), len(dtm), len(spm))
    for part in (nm, dtm, spm):
        body += part + b"\0" * (_pad8(len(part)) - len(part))
    return body + np.ascontiguousarray(a).tobytes()


class _WDataset:
    def __init__(self, data, chunks=None, gzip=None, shuffle=False):
        self.attrs = Attributes()
        self.data = np.array(data, order="C")  # keeps 0-d (scalar) datasets 0-d
        self.chunks, self.gzip, self.shuffle = chunks, gzip, shuffle

    @property
    def shape(self):
        return self.data.shape

    @property
    def dtype(self):
        return self.data.dtype

    def __getitem__(self, key):
        return self.data[key]

    def __setitem__(self, key, value):
        self.data[key] = value


class _WGroup:
    def __init__(self):
        self.attrs = Attributes()
        self.children = {}

    def _walk(self, path, create):
        parts = [p for p in path.split("/") if p]
        node = self
        for part in parts[:-1]:
            nxt = node.children.get(part)
            if nxt is None:
                if not create:
                    raise KeyError(path)
                nxt = node.children[part] = _WGroup()
            if not isinstance(nxt, _WGroup):
                raise KeyError(path)
            node = nxt
        return node, (parts[-1] if parts else None)

    def create_group(self, path):
        parent, leaf = self._walk(path, True)
        if leaf in parent.children:
            raise ValueError("%s exists" % path)
        g = parent.children[leaf] = _WGroup()
        return g

    def require_group(self, path):
        parent, leaf = self._walk(path, True)
        g = parent.children.get(leaf)
        if g is None:
            g = parent.children[leaf] = _WGroup()
        if not isinstance(g, _WGroup):
            raise TypeError("%s is a dataset" % path)
        return g

    def create_dataset(self, path, shape=None, dtype=None, data=None, chunks=None, compression=None,
                       compression_opts=None, shuffle=False):
        """h5py's create_dataset: ``chunks`` (a tuple, or True for the whole array as one chunk),
        ``compression="gzip"`` with level ``compression_opts`` (default 4), ``shuffle``."""
        if compression not in (None, "gzip"):
            raise NotImplementedError("compression %r" % (compression,))
        if (compression or shuffle) and chunks is None:
            chunks = True
        parent, leaf = self._walk(path, True)
        if leaf in parent.children:
            raise ValueError("%s exists" % path)
        if data is None:
            a = np.zeros(shape, dtype=np.dtype(dtype or "f8"))
        else:
            a = _as_array(data)
            if dtype is not None:
                a = a.astype(np.dtype(dtype))
            if shape is not None and tuple(shape) != a.shape:
                a = a.reshape(shape)
        if chunks is True:
            chunks = tuple(max(1, s) for s in a.shape)
        if chunks is not None:
            chunks = tuple(int(c) for c in chunks)
            if a.ndim == 0 or len(chunks) != a.ndim or min(chunks) < 1:
                raise ValueError("chunks %s do not fit a dataset of shape %s" % (chunks, a.shape))
        level = (4 if compression_opts is None else int(compression_opts)) if compression else None
        ds = parent.children[leaf] = _WDataset(a, chunks, level, bool(shuffle))
        return ds

    def __getitem__(self, path):
        parent, leaf = self._walk(path, False)
        if leaf is None:
            return self
        if leaf not in parent.children:
            raise KeyError(path)
        return parent.children[leaf]

    def __contains__(self, path):
        try:
            self[path]
            return True
        except KeyError:
            return False

    def keys(self):
        return list(self.children.keys())


def _copy_tree(src: Group, dst: _WGroup):
    for k, v in src.attrs.items():
        dst.attrs[k] = v
    for name in src.keys():
        node = src[name]
        if isinstance(node, Group):
            _copy_tree(node, dst.create_group(name))
        else:
            if node.dtype.kind not in "iufS":
                raise NotImplementedError("appending to a file holding %s data" % node.dtype)
            ds = dst.create_dataset(name, data=node[()])
            for k, v in node.attrs.items():
                ds.attrs[k] = v


class _Writer(_WGroup):
    def __init__(self, path, keep=False):
        super().__init__()
        self.path = path
        self._closed = False
        if keep:
            import os

            if os.path.exists(path):
                _copy_tree(File(path), self)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        if exc[0] is None:
            self.close()
        return False

    def close(self):
        if self._closed:
            return
        self._closed = True
        out = bytearray(b"\0" * 96)  # superblock 0 and the root symbol table entry
        root_hdr, root_bt, root_heap = self._emit_group(out, self)
        sb = _SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", _LEAF_K, _INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, _UNDEF, len(out), _UNDEF)
        sb += struct.pack("<QQII", 0, root_hdr, 1, 0) + struct.pack("<QQ", root_bt, root_heap)
        out[0:len(sb)] = sb
        with open(self.path, "wb") as fh:
            fh.write(bytes(out))

    @staticmethod
    def _alloc(out: bytearray, blob: bytes) -> int:
        while len(out) % 8:
            out.append(0)
        a = len(out)
        out += blob
        return a

    def _emit_header(self, out, msgs) -> int:
        body = b"".join(msgs)
        return self._alloc(out, struct.pack("<BBHII", 1, 0, len(msgs), 1, len(body)) + b"\0" * 4 + body)

    def _emit_dataset(self, out, ds: _WDataset) -> int:
        a = ds.data
        msgs = [_message(0x0001, _dataspace_message(a.shape)), _message(0x0003, _dtype_message(a.dtype), 1)]
        if ds.chunks is None:
            addr = self._alloc(out, a.tobytes()) if a.nbytes else _UNDEF
            msgs.append(_message(0x0008, bytes([3, 1]) + struct.pack("<QQ", addr, a.nbytes)))
        else:
            filters = []
            if ds.shuffle:
                filters.append((2, [a.dtype.itemsize]))
            if ds.gzip is not None:
                filters.append((1, [ds.gzip]))
            if filters:  # filter pipeline message, version 1
                body = bytes([1, len(filters)]) + bytes(6)
                for fid, vals in filters:
                    body += struct.pack("<HHHH", fid, 0, 0, len(vals)) + b"".join(struct.pack("<I", v) for v in vals)
                    if len(vals) % 2:
                        body += bytes(4)
                msgs.append(_message(0x000B, body))
            bt = self._emit_chunks(out, a, ds.chunks, filters)
            lay = bytes([3, 2, a.ndim + 1]) + struct.pack("<Q", bt)
            lay += b"".join(struct.pack("<I", c) for c in ds.chunks) + struct.pack("<I", a.dtype.itemsize)
            msgs.append(_message(0x0008, lay))
        msgs += [_message(0x000C, _attribute_message(k, v)) for k, v in ds.attrs.items()]
        return self._emit_header(out, msgs)

    _CHUNK_K = 32  # libhdf5's default "indexed storage internal node K": 2K entries per node

    def _emit_chunks(self, out, a, chunks, filters) -> int:
        """Write every chunk (edge chunks zero-filled to full size, filtered) and a B-tree v1 chunk
        index over them (node type 1, keys: stored size, filter mask, element offsets)."""
        rank = a.ndim
        grid = [-(-s // c) for s, c in zip(a.shape, chunks)]
        entries = []  # (key bytes, child address)
        for idx in np.ndindex(*grid):
            offs = [i * c for i, c in zip(idx, chunks)]
            blk = np.zeros(chunks, dtype=a.dtype)
            src = a[tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, chunks, a.shape))]
            blk[tuple(slice(0, n) for n in src.shape)] = src
            raw = blk.tobytes()
            for fid, vals in filters:
                if fid == 2:  # shuffle: byte k of every element together
                    es = vals[0]
                    raw = np.frombuffer(raw, dtype=np.uint8).reshape(-1, es).T.tobytes()
                elif fid == 1:
                    raw = zlib.compress(raw, vals[0])
            addr = self._alloc(out, raw)
            entries.append((struct.pack("<II", len(raw), 0) + b"".join(struct.pack("<Q", o) for o in offs + [0]), addr))
        end_key = struct.pack("<II", 0, 0) + b"".join(struct.pack("<Q", g * c) for g, c in zip(grid, chunks)) + bytes(8)
        ksize = 8 + 8 * (rank + 1)
        cap = 2 * self._CHUNK_K
        level = 0
        while True:
            nodes = []
            for i in range(0, len(entries), cap):
                part = entries[i:i + cap]
                last = entries[i + cap][0] if i + cap < len(entries) else end_key
                blob = b"TREE" + bytes([1, level]) + struct.pack("<HQQ", len(part), _UNDEF, _UNDEF)
                for key, child in part:
                    blob += key + struct.pack("<Q", child)
                blob += last
                blob += bytes(24 + cap * 8 + (cap + 1) * ksize - len(blob))
                nodes.append((part[0][0], self._alloc(out, blob)))
            if len(nodes) == 1:
                return nodes[0][1]
            entries, level = nodes, level + 1

    def _emit_group(self, out, g: _WGroup):
        names = sorted(g.children.keys(), key=lambda s: s.encode())  # symbol nodes are searched by name
        if len(names) > 2 * _LEAF_K * 2 * _INTERNAL_K:
            raise NotImplementedError("more than %d members in one group" % (4 * _LEAF_K * _INTERNAL_K))
        entries = []
        for nm in names:
            ch = g.children[nm]
            if isinstance(ch, _WGroup):
                h, bt, hp = self._emit_group(out, ch)
                entries.append((nm, h, 1, bt, hp))
            else:
                entries.append((nm, self._emit_dataset(out, ch), 0, 0, 0))
        # local heap: "" at offset 0, the names 8-aligned after it, then one free block (next
        # offset 1 = end of the free list, and its size), as libhdf5 lays it out
        heap_data = bytearray(b"\0" * 8)
        offs = {}
        for nm in names:
            offs[nm] = len(heap_data)
            s = nm.encode() + b"\0"
            heap_data += s + b"\0" * (_pad8(len(s)) - len(s))
        free_off = len(heap_data)
        heap_data += struct.pack("<QQ", 1, 16)
        data_addr = self._alloc(out, bytes(heap_data))
        heap_addr = self._alloc(out, b"HEAP" + bytes(4) + struct.pack("<QQQ", len(heap_data), free_off, data_addr))
        # symbol nodes of up to 2*LEAF_K entries; key i+1 = name offset of child i's last entry
        snods, keys = [], [0]
        for i in range(0, len(entries), 2 * _LEAF_K):
            chunk = entries[i:i + 2 * _LEAF_K]
            blob = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(chunk))
            for nm, h, ct, bt, hp in chunk:
                blob += struct.pack("<QQII", offs[nm], h, ct, 0) + struct.pack("<QQ", bt, hp)
            blob += b"\0" * (8 + 2 * _LEAF_K * 40 - len(blob))
            snods.append(self._alloc(out, blob))
            keys.append(offs[chunk[-1][0]])
        bt = b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", len(snods), _UNDEF, _UNDEF)
        for i, s in enumerate(snods):
            bt += struct.pack("<QQ", keys[i], s)
        bt += struct.pack("<Q", keys[len(snods)])
        bt += b"\0" * (24 + 2 * _INTERNAL_K * 8 + (2 * _INTERNAL_K + 1) * 8 - len(bt))
        bt_addr = self._alloc(out, bt)
        msgs = [_message(0x0011, struct.pack("<QQ", bt_addr, heap_addr))]
        msgs += [_message(0x000C, _attribute_message(k, v)) for k, v in g.attrs.items()]
        return self._emit_header(out, msgs), bt_addr, heap_addr
