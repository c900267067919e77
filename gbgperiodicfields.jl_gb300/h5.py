"""HDF5 files without an HDF5 library: a reader and a writer of the file format itself,
written from the public HDF5 File Format Specification (version 3.0), for the
checkpoints of ``checkpoint.py``.

The reference persists fields, point sets and transfer schemes through HDF5.jl
(ext/GBGPeriodicFieldsHDF5Ext.jl); neither libhdf5 nor h5py is available to this
package, so the format is implemented here.  What is covered:

* reading: superblocks 0-3 (a user block before the superblock is found by the
  signature search at 0, 512, 1024, ...), version 1 and 2 object headers with their
  continuation blocks, groups stored as symbol tables (v1 B-tree + local heap), as
  compact link messages, or densely (fractal heap + v2 B-tree of link names),
  attributes in object headers or densely, contiguous and compact datasets (chunked
  ones with the version 1 B-tree chunk index, unfiltered or deflate-compressed), the
  fixed-point, floating-point, string, compound (a pair r/i of floats reads as
  complex), enum, and variable-length string types; every checksum is verified;
* writing: superblock version 2, version 2 object headers, compact links and
  attributes, contiguous datasets, and chunked ones on request (a version 1 B-tree of
  chunk records, up to 64 a node, each chunk optionally deflated), the same datatypes
  as the reader (strings as fixed-length UTF-8, complex as the compound {r, i} HDF5.jl
  uses), to the version of the specification libhdf5 1.8 and later read.  No libhdf5
  is at hand to open the results, so writing is checked against this module's reader,
  which is itself pinned to files libhdf5 wrote (contiguous ones: HDF5.jl, MATLAB and
  the default here store datasets contiguously, and no chunked file written by libhdf5
  is at hand, so the chunked layout is checked by round trips alone).

Arrays follow Julia's (and HDF5.jl's) convention: an array of shape S, column-major,
is stored as the dataspace reversed(S) over the same bytes, so a file written here
reads in Julia with the shape it was written with, and vice versa.  In Python the
array comes back as a Fortran-ordered numpy array of shape S.

A file opened for writing ("w") or modification ("r+", "a") is held as a tree of
groups, datasets and attributes; closing it writes the whole tree to a fresh file
(the data of datasets that came from the old file is copied from it) and moves the
fresh file into place.
"""
from __future__ import annotations

import os
import struct
import tempfile
import zlib
from collections.abc import MutableMapping

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(ValueError):
    """A file this module cannot read: malformed, or using a feature outside its scope."""


# ---------------------------------------------------------------------------- checksum


def _rot(x, k):
    return ((x << k) | (x >> (32 - k))) & 0xFFFFFFFF


def lookup3(data: bytes, initval: int = 0) -> int:
    """Bob Jenkins' lookup3 hash (hashlittle, 2006, public domain), the checksum of the
    HDF5 format's version 2 metadata: 32-bit words a, b, c mixed over 12-byte blocks,
    the last (partial) block added byte-wise and finished by the final mix."""
    M = 0xFFFFFFFF
    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & M
    i = 0
    while n - i > 12:
        a = (a + int.from_bytes(data[i:i + 4], "little")) & M
        b = (b + int.from_bytes(data[i + 4:i + 8], "little")) & M
        c = (c + int.from_bytes(data[i + 8:i + 12], "little")) & M
        a = (a - c) & M; a ^= _rot(c, 4); c = (c + b) & M
        b = (b - a) & M; b ^= _rot(a, 6); a = (a + c) & M
        c = (c - b) & M; c ^= _rot(b, 8); b = (b + a) & M
        a = (a - c) & M; a ^= _rot(c, 16); c = (c + b) & M
        b = (b - a) & M; b ^= _rot(a, 19); a = (a + c) & M
        c = (c - b) & M; c ^= _rot(b, 4); b = (b + a) & M
        i += 12
    rest = n - i
    if rest == 0:
        return c
    tail = data[i:] + bytes(12 - rest)
    a = (a + int.from_bytes(tail[0:4], "little")) & M
    b = (b + int.from_bytes(tail[4:8], "little")) & M
    c = (c + int.from_bytes(tail[8:12], "little")) & M
    c ^= b; c = (c - _rot(b, 14)) & M
    a ^= c; a = (a - _rot(c, 11)) & M
    b ^= a; b = (b - _rot(a, 25)) & M
    c ^= b; c = (c - _rot(b, 16)) & M
    a ^= c; a = (a - _rot(c, 4)) & M
    b ^= a; b = (b - _rot(a, 14)) & M
    c ^= b; c = (c - _rot(b, 24)) & M
    return c


def _bytes_for(value: int) -> int:
    """Bytes needed to encode the unsigned value (at least 1)."""
    return max(1, (int(value).bit_length() + 7) // 8)


# ---------------------------------------------------------------------------- datatypes


class Datatype:
    """A decoded HDF5 datatype.  kind: 'int', 'float', 'string', 'vlen_string',
    'compound', 'complex', 'enum', 'opaque' or 'bitfield'; dtype: the numpy dtype of one
    stored element (for 'vlen_string' the 16-byte heap reference)."""

    def __init__(self, kind, size, dtype, **extra):
        self.kind = kind
        self.size = size
        self.dtype = np.dtype(dtype)
        self.__dict__.update(extra)


def _decode_datatype(buf, off):
    """Datatype message (format spec IV.A.2.d) at buf[off:]; returns (Datatype, end)."""
    cv, b0, b1, b2 = buf[off], buf[off + 1], buf[off + 2], buf[off + 3]
    cls, version = cv & 0x0F, cv >> 4
    size = struct.unpack_from("<I", buf, off + 4)[0]
    p = off + 8
    if cls == 0:  # fixed-point
        order = ">" if b0 & 1 else "<"
        signed = bool(b0 & 0x08)
        p += 4
        if size not in (1, 2, 4, 8):
            raise H5Error(f"integer of {size} bytes")
        return Datatype("int", size, f"{order}{'i' if signed else 'u'}{size}"), p
    if cls == 1:  # floating-point
        if b0 & 0x40:
            raise H5Error("VAX floating-point order")
        order = ">" if b0 & 1 else "<"
        p += 12
        if size not in (2, 4, 8):
            raise H5Error(f"floating-point of {size} bytes")
        return Datatype("float", size, f"{order}f{size}"), p
    if cls == 2:  # time (obsolete): opaque integers
        p += 2
        return Datatype("opaque", size, f"V{size}"), p
    if cls == 3:  # string
        return Datatype("string", size, f"S{size}", pad=b0 & 0x0F, cset=b0 >> 4), p
    if cls == 4:  # bitfield
        p += 4
        return Datatype("bitfield", size, f"V{size}"), p
    if cls == 5:  # opaque: an ASCII tag padded to 8 bytes
        p += b0
        return Datatype("opaque", size, f"V{size}"), p
    if cls == 6:  # compound
        nmembers = b0 | (b1 << 8)
        names, offsets, types = [], [], []
        for _ in range(nmembers):
            end = buf.index(b"\0", p)
            name = bytes(buf[p:end]).decode("utf-8")
            if version < 3:
                p += ((end - p) // 8 + 1) * 8
                moff = struct.unpack_from("<I", buf, p)[0]
                p += 4
                if version == 1:
                    ndims = buf[p]
                    p += 1 + 3 + 4 + 4 + 16
                    if ndims:
                        raise H5Error("compound member with array dimensions")
            else:
                p = end + 1
                nb = _bytes_for(size) if size else 1
                moff = int.from_bytes(buf[p:p + nb], "little")
                p += nb
            mt, p = _decode_datatype(buf, p)
            names.append(name)
            offsets.append(moff)
            types.append(mt)
        pair = [n.lower() for n in names]
        if (nmembers == 2 and pair in (["r", "i"], ["re", "im"], ["real", "imag"]) and types[0].kind == "float"
                and types[1].kind == "float" and types[0].size == types[1].size and offsets == [0, types[0].size]
                and size == 2 * types[0].size):
            order = types[0].dtype.str[0]
            return Datatype("complex", size, f"{order}c{size}"), p
        fields = {"names": names, "formats": [t.dtype for t in types], "offsets": offsets, "itemsize": size}
        return Datatype("compound", size, np.dtype(fields), members=list(zip(names, types))), p
    if cls == 8:  # enum: base type, then names and values
        nmembers = b0 | (b1 << 8)
        base, p = _decode_datatype(buf, p)
        names = []
        for _ in range(nmembers):
            end = buf.index(b"\0", p)
            names.append(bytes(buf[p:end]).decode("utf-8"))
            p = end + 1 if version >= 3 else p + ((end - p) // 8 + 1) * 8
        values = [int.from_bytes(buf[p + i * base.size:p + (i + 1) * base.size], "little") for i in range(nmembers)]
        p += nmembers * base.size
        return Datatype("enum", size, base.dtype, names=dict(zip(values, names))), p
    if cls == 9:  # variable-length
        vtype = b0 & 0x0F
        base, p = _decode_datatype(buf, p)
        if vtype == 1:
            return Datatype("vlen_string", size, "V16", pad=(b0 >> 4) & 0x0F, cset=b1 & 0x0F), p
        return Datatype("vlen", size, "V16", base=base), p
    raise H5Error(f"datatype class {cls} is not supported")


def _float_props(size):
    if size == 8:
        return struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023), 63
    if size == 4:
        return struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127), 31
    if size == 2:
        return struct.pack("<HHBBBBI", 0, 16, 10, 5, 0, 10, 15), 15
    raise H5Error(f"no HDF5 encoding for a float of {size} bytes")


def _encode_datatype(dt: np.dtype) -> bytes:
    """Datatype message (version 1) for a numpy dtype: little-endian integers and IEEE
    floats, complex as the compound {r, i}, and fixed-length UTF-8 strings ('S' dtypes,
    null-terminated as HDF5.jl writes them)."""
    dt = np.dtype(dt)
    if dt.kind in "iu":
        b0 = 0x08 if dt.kind == "i" else 0
        return struct.pack("<BBBBI", 0x10 | 0, b0, 0, 0, dt.itemsize) + struct.pack("<HH", 0, 8 * dt.itemsize)
    if dt.kind == "b":
        return _encode_datatype(np.dtype("u1"))
    if dt.kind == "f":
        props, sign = _float_props(dt.itemsize)
        return struct.pack("<BBBBI", 0x10 | 1, 0x20, sign, 0, dt.itemsize) + props
    if dt.kind == "c":
        half = dt.itemsize // 2
        member = _encode_datatype(np.dtype(f"<f{half}"))
        body = b""
        for name, moff in ((b"r", 0), (b"i", half)):
            body += name + b"\0" * (8 - len(name)) + struct.pack("<IB3sI4s16s", moff, 0, b"", 0, b"", b"") + member
        return struct.pack("<BBBBI", 0x10 | 6, 2, 0, 0, dt.itemsize) + body
    if dt.kind == "S":
        return struct.pack("<BBBBI", 0x10 | 3, 0x10 | 0, 0, 0, max(dt.itemsize, 1))
    raise H5Error(f"no HDF5 encoding for numpy dtype {dt}")


# ---------------------------------------------------------------------------- dataspaces


def _decode_dataspace(buf, off):
    """Dataspace message at buf[off:]; returns the dims in HDF5 (C, slowest first) order,
    () for a scalar, or None for a null dataspace."""
    version, ndims, flags = buf[off], buf[off + 1], buf[off + 2]
    if version == 1:
        p = off + 8
        kind = 1 if ndims else 0
    elif version == 2:
        kind = buf[off + 3]
        p = off + 4
    else:
        raise H5Error(f"dataspace message version {version}")
    dims = struct.unpack_from(f"<{ndims}Q", buf, p) if ndims else ()
    if kind == 2:
        return None
    return tuple(int(d) for d in dims)


def _encode_dataspace(dims) -> bytes:
    if dims is None:
        return struct.pack("<BBBB", 2, 0, 0, 2)
    if len(dims) == 0:
        return struct.pack("<BBBB", 2, 0, 0, 0)
    return struct.pack("<BBBB", 2, len(dims), 0, 1) + struct.pack(f"<{len(dims)}Q", *dims)


# ---------------------------------------------------------------------------- values


def _to_value(raw: bytes, dtype: Datatype, dims, reader=None):
    """Decoded stored bytes as a Python/numpy value: a scalar for a scalar dataspace,
    else an array of shape reversed(dims) in Fortran order (Julia's view of it)."""
    if dims is None:
        return None
    count = int(np.prod(dims)) if dims else 1
    if dtype.kind == "vlen_string":
        refs = np.frombuffer(raw, dtype=np.dtype([("n", "<u4"), ("addr", "<u8"), ("idx", "<u4")]), count=count)
        items = [reader.global_heap_object(int(r["addr"]), int(r["idx"]))[: int(r["n"])].decode("utf-8", "replace")
                 if int(r["addr"]) not in (0, UNDEF) else "" for r in refs]
        if not dims:
            return items[0]
        return np.array(items, dtype=object).reshape(tuple(reversed(dims)), order="F")
    arr = np.frombuffer(raw, dtype=dtype.dtype, count=count)
    if dtype.kind == "string":
        strip = b" " if dtype.pad == 2 else b"\0"
        out = [s.split(b"\0", 1)[0].rstrip(strip).decode("utf-8", "replace") for s in arr.tolist()]
        if not dims:
            return out[0]
        return np.array(out, dtype=object).reshape(tuple(reversed(dims)), order="F")
    if dtype.dtype.byteorder == ">":
        arr = arr.astype(dtype.dtype.newbyteorder("<"))
    if not dims:
        v = arr[0]
        return v.item() if dtype.kind in ("int", "float", "complex", "enum") else v
    return arr.reshape(tuple(reversed(dims)), order="F").copy(order="F")  # writable


def _from_value(value):
    """(numpy dtype, HDF5 dims or (), raw bytes) of a value to store.  str -> fixed UTF-8
    string; Python int/float/complex/bool -> int64/float64/complex128/uint8 scalar;
    numpy scalars keep their type; arrays are taken in Julia's (Fortran) order."""
    if isinstance(value, str):
        raw = value.encode("utf-8")
        return np.dtype(f"S{max(len(raw), 1)}"), (), raw if raw else b"\0"
    if isinstance(value, (bool, np.bool_)):
        return np.dtype("u1"), (), bytes([1 if value else 0])
    if isinstance(value, int):
        return np.dtype("<i8"), (), struct.pack("<q", value)
    if isinstance(value, float):
        return np.dtype("<f8"), (), struct.pack("<d", value)
    if isinstance(value, complex):
        return np.dtype("<c16"), (), struct.pack("<dd", value.real, value.imag)
    if isinstance(value, np.generic):
        a = np.asarray(value)
        return a.dtype.newbyteorder("<"), (), a.astype(a.dtype.newbyteorder("<")).tobytes()
    a = np.asarray(value)
    if a.dtype.kind in "UO":
        enc = [str(s).encode("utf-8") for s in a.ravel(order="F")]
        width = max([len(e) for e in enc] + [1])
        a = np.array(enc, dtype=f"S{width}").reshape(a.shape, order="F")
    if a.dtype.kind not in "iufcSb":
        raise H5Error(f"cannot store values of dtype {a.dtype}")
    if a.dtype.kind != "S" and a.dtype.byteorder == ">":
        a = a.astype(a.dtype.newbyteorder("<"))
    return a.dtype, tuple(reversed(a.shape)), None


# ---------------------------------------------------------------------------- tree


class Attributes(MutableMapping):
    """The attributes of a group or dataset, in creation order."""

    def __init__(self, owner):
        self._owner = owner
        self._items = {}

    def __getitem__(self, name):
        return self._items[name]

    def __setitem__(self, name, value):
        self._owner._file._writable()
        _from_value(value)  # refuse unstorable values at once
        self._items[name] = value.item() if isinstance(value, np.ndarray) and value.ndim == 0 else value

    def __delitem__(self, name):
        self._owner._file._writable()
        del self._items[name]

    def __iter__(self):
        return iter(self._items)

    def __len__(self):
        return len(self._items)


class Node:
    def __init__(self, file, name):
        self._file = file
        self.name = name
        self.attrs = Attributes(self)


class Dataset(Node):
    """A dataset: shape (Julia's, column-major; () for a scalar), numpy dtype, and data
    in the file it was read from, or (once created) in the file being written."""

    def __init__(self, file, name, dtype, shape, value=None, stored=None, written=None):
        super().__init__(file, name)
        self.dtype = dtype
        self.shape = shape
        self._value = value      # a scalar or string value, kept as given
        self._stored = stored    # (reader, Datatype, HDF5 dims, layout) in the file read
        self._written = written  # (address, byte count, numpy dtype, HDF5 dims) in the output
        # a chunked dataset written here: {"chunk": HDF5-order chunk dims, "level": deflate
        # level or None, "entries": [(HDF5 offsets, address, bytes), ...]}; the address in
        # _written is then its chunk B-tree's
        self._chunked = None

    @property
    def ndim(self):
        return len(self.shape) if self.shape is not None else 0

    def read(self):
        if self._value is not None:
            return self._value
        if self._written is not None and self._chunked is not None:
            _, _, dt, dims = self._written
            c = self._chunked
            full = np.zeros(tuple(dims), dtype=dt)
            for offs, caddr, n in c["entries"]:
                raw = self._file._read_output(caddr, n)
                if c["level"] is not None:
                    raw = zlib.decompress(raw)
                block = np.frombuffer(raw, dtype=dt).reshape(c["chunk"])
                sl = tuple(slice(o, min(o + k, d)) for o, k, d in zip(offs, c["chunk"], dims))
                full[sl] = block[tuple(slice(0, q.stop - q.start) for q in sl)]
            return np.asfortranarray(full.T)
        if self._written is not None:
            addr, nbytes, dt, dims = self._written
            raw = self._file._read_output(addr, nbytes)
            if dt.kind == "S":
                return _to_value(raw, Datatype("string", dt.itemsize, dt, pad=0, cset=1), dims)
            return np.frombuffer(raw, dtype=dt).reshape(tuple(reversed(dims)), order="F").copy()
        reader, dt, dims, layout = self._stored
        if dims and dt.kind in ("int", "float", "complex") and dt.dtype.byteorder != ">":
            out = np.empty(tuple(reversed(dims)), dtype=dt.dtype, order="F")  # one read, no staging copy
            reader.dataset_into(layout, dt, dims, out.T.reshape(-1).view(np.uint8) if out.ndim > 1 else out.view(np.uint8))
            return out
        return _to_value(reader.dataset_bytes(layout, dt, dims), dt, dims, reader)

    def read_into(self, out: np.ndarray):
        """Reads a numeric dataset straight into a Fortran-contiguous array of its shape
        and dtype (read_field!'s copy-free path)."""
        if tuple(out.shape) != tuple(self.shape) or np.dtype(out.dtype) != np.dtype(self.dtype):
            raise H5Error(f"read_into: destination {out.dtype}{tuple(out.shape)} but dataset {self.dtype}{self.shape}")
        if not out.flags.f_contiguous:
            raise H5Error("read_into: destination must be Fortran-contiguous")
        flat = out.T.reshape(-1) if out.ndim > 1 else out.reshape(-1)
        if self._stored is not None and self._written is None:
            reader, dt, dims, layout = self._stored
            if dt.kind in ("int", "float", "complex") and dt.dtype.byteorder != ">":
                reader.dataset_into(layout, dt, dims, flat.view(np.uint8))
                return out
        v = np.asarray(self.read())
        flat[...] = v.T.reshape(-1) if v.ndim > 1 else v.reshape(-1)
        return out


class Group(Node):
    """A group: named links to groups and datasets, and attributes."""

    def __init__(self, file, name):
        super().__init__(file, name)
        self._links = {}

    def _resolve(self, path):
        node = self
        for part in [p for p in path.split("/") if p]:
            if not isinstance(node, Group) or part not in node._links:
                raise KeyError(path)
            node = node._links[part]
        return node

    def __getitem__(self, path):
        return self._resolve(path)

    def __contains__(self, path):
        try:
            self._resolve(path)
            return True
        except KeyError:
            return False

    def keys(self):
        return list(self._links)

    def __iter__(self):
        return iter(self._links)

    def __len__(self):
        return len(self._links)

    def _parent_and_leaf(self, path):
        parts = [p for p in path.split("/") if p]
        if not parts:
            raise KeyError("empty name")
        parent = self._resolve("/".join(parts[:-1])) if len(parts) > 1 else self
        if not isinstance(parent, Group):
            raise KeyError(path)
        return parent, parts[-1]

    def create_group(self, path) -> "Group":
        self._file._writable()
        parent, leaf = self._parent_and_leaf(path)
        if leaf in parent._links:
            raise H5Error(f"an object named {path!r} already exists")
        g = Group(self._file, leaf)
        parent._links[leaf] = g
        return g

    def require_group(self, path) -> "Group":
        return self[path] if path in self else self.create_group(path)

    def create_dataset(self, path, value, chunks=None, compression=None) -> Dataset:
        """A dataset holding value.  A numeric array may be stored in chunks (`chunks`, one
        extent per axis in the array's own, Julia, order; edge chunks are stored whole) and
        each chunk deflate-compressed (`compression`, a zlib level 0-9, chunked only);
        otherwise the data is one contiguous block."""
        self._file._writable()
        parent, leaf = self._parent_and_leaf(path)
        if leaf in parent._links:
            raise H5Error(f"an object named {path!r} already exists")
        dt, dims, raw = _from_value(value)
        if compression is not None and chunks is None:
            raise H5Error("compression needs a chunked layout (chunks=...)")
        if chunks is not None:
            a = np.asarray(value)
            chunks = tuple(int(c) for c in chunks)
            if raw is not None or dt.kind not in "biufc" or a.ndim == 0 or a.size == 0:
                raise H5Error("chunks: only non-empty numeric arrays are stored in chunks")
            if len(chunks) != a.ndim or any(c < 1 for c in chunks):
                raise H5Error(f"chunks: {len(chunks)} extents >= 1 expected for an array of {a.ndim} axes")
            if compression is not None and not 0 <= int(compression) <= 9:
                raise H5Error("compression: a deflate level 0-9")
            level = None if compression is None else int(compression)
            btree, nbytes, entries, cdims = self._file._append_chunked(a, dt, chunks, level)
            ds = Dataset(self._file, leaf, dt, tuple(a.shape), written=(btree, nbytes, dt, dims))
            ds._chunked = {"chunk": cdims, "level": level, "entries": entries}
        elif raw is not None:
            ds = Dataset(self._file, leaf, dt, (), value=value)
        else:
            a = np.asarray(value)
            # the bytes go to the output now, as HDF5 writes them: later changes to the
            # array do not reach the file, and nothing is copied on the way
            addr, nbytes = self._file._append(a, dt)
            ds = Dataset(self._file, leaf, np.dtype(object) if dt.kind == "S" else dt, tuple(a.shape),
                         written=(addr, nbytes, dt, dims))
        parent._links[leaf] = ds
        return ds

    def __setitem__(self, path, value):
        writer = getattr(value, "_h5_write", None)
        if writer is not None:
            writer(self, path)
            return
        from . import checkpoint  # the sugar parent[name] = field / points / scheme
        if checkpoint.write_object(self, path, value):
            return
        self.create_dataset(path, value)

    def __delitem__(self, path):
        self._file._writable()
        parent, leaf = self._parent_and_leaf(path)
        if leaf not in parent._links:
            raise KeyError(path)
        del parent._links[leaf]


# ---------------------------------------------------------------------------- reader


class _Reader:
    """Parses an existing file into the tree; keeps the file open for lazy data reads."""

    def __init__(self, path):
        self.f = open(path, "rb")
        self.size = os.fstat(self.f.fileno()).st_size
        self._gheaps = {}
        base = None
        for cand in [0] + [512 << k for k in range(0, 40)]:
            if cand + 8 > self.size:
                break
            self.f.seek(cand)
            if self.f.read(8) == SIGNATURE:
                base = cand
                break
        if base is None:
            raise H5Error(f"{path}: no HDF5 signature")
        self.sb_at = base
        sb = self.raw(base, 256)
        version = sb[8]
        if version in (0, 1):
            self.O, self.L = sb[13], sb[14]
            p = 24 + (4 if version == 1 else 0)
            if self.O != 8 or self.L != 8:
                raise H5Error("only 8-byte offsets and lengths are supported")
            self.base, _free, self.eof, _drv = struct.unpack_from("<4Q", sb, p)
            p += 32
            _name_off, self.root_addr = struct.unpack_from("<QQ", sb, p)
        elif version in (2, 3):
            self.O, self.L = sb[9], sb[10]
            if self.O != 8 or self.L != 8:
                raise H5Error("only 8-byte offsets and lengths are supported")
            self.base, _ext, self.eof, self.root_addr = struct.unpack_from("<4Q", sb, 12)
            self._check(sb[:44], struct.unpack_from("<I", sb, 44)[0], "superblock")
        else:
            raise H5Error(f"superblock version {version}")
        self.sb_version = version

    def close(self):
        self.f.close()

    def raw(self, addr, n):
        self.f.seek(addr)
        return self.f.read(n)

    def at(self, addr, n):
        """n bytes at a file address (relative to the base address)."""
        b = self.raw(self.base + addr, n)
        if len(b) < n:
            raise H5Error(f"read past the end of the file at {addr}")
        return b

    @staticmethod
    def _check(data, want, what):
        got = lookup3(bytes(data))
        if got != want:
            raise H5Error(f"checksum mismatch in {what}: stored {want:#010x}, computed {got:#010x}")

    # ---- object headers

    def messages(self, addr):
        """The (type, flags, data) messages of the object header at addr."""
        head = self.at(addr, 16)
        out = []
        if head[:4] == b"OHDR":
            version, flags = head[4], head[5]
            if version != 2:
                raise H5Error(f"object header version {version}")
            p = 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
            nb = 1 << (flags & 3)
            pre = self.at(addr, p + nb)
            size0 = int.from_bytes(pre[p:p + nb], "little")
            block = self.at(addr, p + nb + size0 + 4)
            self._check(block[:-4], struct.unpack_from("<I", block, len(block) - 4)[0], "object header")
            pending = [(block, p + nb, p + nb + size0)]
            creation = bool(flags & 0x04)
            while pending:
                blk, s, e = pending.pop(0)
                q = s
                hsize = 6 if creation else 4
                while q + hsize <= e:
                    mtype, msize, mflags = blk[q], struct.unpack_from("<H", blk, q + 1)[0], blk[q + 3]
                    q += hsize
                    data = blk[q:q + msize]
                    q += msize
                    if mtype == 0x10:
                        caddr, clen = struct.unpack_from("<QQ", data, 0)
                        cblk = self.at(caddr, clen)
                        if cblk[:4] != b"OCHK":
                            raise H5Error("bad continuation block signature")
                        self._check(cblk[:-4], struct.unpack_from("<I", cblk, clen - 4)[0], "continuation block")
                        pending.append((cblk, 4, clen - 4))
                    else:
                        out.append((mtype, mflags, data))
        else:
            version = head[0]
            if version != 1:
                raise H5Error(f"unknown object header at {addr}")
            nmsg, _refs, hsize = struct.unpack_from("<HII", head, 2)
            pending = [(self.at(addr + 16, hsize), 0, hsize)]
            seen = 0
            while pending and seen < nmsg:
                blk, s, e = pending.pop(0)
                q = s
                while q + 8 <= e and seen < nmsg:
                    mtype, msize, mflags = struct.unpack_from("<HHB", blk, q)
                    q += 8
                    data = blk[q:q + msize]
                    q += msize
                    seen += 1
                    if mtype == 0x10:
                        caddr, clen = struct.unpack_from("<QQ", data, 0)
                        pending.append((self.at(caddr, clen), 0, clen))
                    else:
                        out.append((mtype, mflags, data))
        for mtype, mflags, _ in out:
            if mflags & 0x02:
                raise H5Error("shared object header messages are not supported")
        return out

    # ---- objects

    def load(self, file, addr, name, cache):
        if addr in cache:
            return cache[addr]
        msgs = self.messages(addr)
        types = {m[0] for m in msgs}
        if 0x08 in types:  # data layout: a dataset
            node = self._dataset(file, name, msgs)
            cache[addr] = node
        else:
            node = Group(file, name)
            cache[addr] = node
            for lname, laddr in self._links(msgs):
                if laddr is None:
                    continue  # soft or external link: not followed
                node._links[lname] = self.load(file, laddr, lname, cache)
        for aname, value in self._attributes(msgs):
            node.attrs._items[aname] = value
        return node

    def _dataset(self, file, name, msgs):
        dt = dims = layout = None
        filters = []
        for mtype, _, data in msgs:
            if mtype == 0x01:
                dims = _decode_dataspace(data, 0)
            elif mtype == 0x03:
                dt, _ = _decode_datatype(data, 0)
            elif mtype == 0x08:
                layout = self._layout(data)
            elif mtype == 0x0B:
                filters = self._filters(data)
        if dt is None or layout is None:
            raise H5Error(f"dataset {name!r} lacks its datatype or layout")
        layout["filters"] = filters
        shape = tuple(reversed(dims)) if dims else (() if dims == () else None)
        npdt = np.dtype(object) if dt.kind in ("string", "vlen_string") else (
            dt.dtype.newbyteorder("<") if dt.dtype.byteorder == ">" else dt.dtype)
        return Dataset(file, name, npdt, shape, stored=(self, dt, dims, layout))

    def _layout(self, data):
        version = data[0]
        if version == 3 or version == 4:
            cls = data[1]
            if cls == 0:
                n = struct.unpack_from("<H", data, 2)[0]
                return {"class": "compact", "data": bytes(data[4:4 + n])}
            if cls == 1:
                addr, size = struct.unpack_from("<QQ", data, 2)
                return {"class": "contiguous", "addr": addr, "size": size}
            if cls == 2 and version == 3:
                nd = data[2]
                addr = struct.unpack_from("<Q", data, 3)[0]
                cdims = struct.unpack_from(f"<{nd}I", data, 11)
                return {"class": "chunked", "addr": addr, "chunk": cdims[:-1], "elem": cdims[-1]}
            raise H5Error(f"data layout class {cls} (message version {version}) is not supported")
        if version in (1, 2):
            nd, cls = data[1], data[2]
            p = 8
            addr = None
            if cls != 0:
                addr = struct.unpack_from("<Q", data, p)[0]
                p += 8
            dims = struct.unpack_from(f"<{nd}I", data, p)
            p += 4 * nd
            if cls == 0:
                n = struct.unpack_from("<I", data, p)[0]
                return {"class": "compact", "data": bytes(data[p + 4:p + 4 + n])}
            if cls == 1:
                return {"class": "contiguous", "addr": addr, "size": None}
            return {"class": "chunked", "addr": addr, "chunk": dims[:-1], "elem": dims[-1]}
        raise H5Error(f"data layout message version {version}")

    def _filters(self, data):
        version, n = data[0], data[1]
        p = 8 if version == 1 else 2
        out = []
        for _ in range(n):
            fid = struct.unpack_from("<H", data, p)[0]
            if version == 1 or fid >= 256:
                name_len = struct.unpack_from("<H", data, p + 2)[0]
                _flags, ncv = struct.unpack_from("<HH", data, p + 4)
                p += 8 + (((name_len + 7) // 8) * 8 if version == 1 else name_len)
            else:
                _flags, ncv = struct.unpack_from("<HH", data, p + 2)
                p += 6
            p += 4 * ncv + (4 if version == 1 and ncv % 2 else 0)
            out.append(fid)
        return out

    def _attributes(self, msgs):
        for mtype, _, data in msgs:
            if mtype == 0x0C:
                yield self._attribute(data)
            elif mtype == 0x15:
                yield from self._dense_attributes(data)

    def _attribute(self, data):
        version = data[0]
        name_size, dt_size, ds_size = struct.unpack_from("<HHH", data, 2)
        if version == 1:
            p = 8
            pad = lambda n: (n + 7) // 8 * 8
        elif version in (2, 3):
            p = 8 + (1 if version == 3 else 0)
            pad = lambda n: n
        else:
            raise H5Error(f"attribute message version {version}")
        name = bytes(data[p:p + name_size]).split(b"\0", 1)[0].decode("utf-8")
        p += pad(name_size)
        dt, _ = _decode_datatype(data, p)
        p += pad(dt_size)
        dims = _decode_dataspace(data, p)
        p += pad(ds_size)
        count = int(np.prod(dims)) if dims else (1 if dims == () else 0)
        raw = bytes(data[p:p + count * dt.size])
        return name, _to_value(raw, dt, dims, self)

    def _links(self, msgs):
        for mtype, _, data in msgs:
            if mtype == 0x06:
                yield self._link(data)
            elif mtype == 0x11:
                btree, heap = struct.unpack_from("<QQ", data, 0)
                yield from self._symbol_table(btree, heap)
            elif mtype == 0x02:
                flags = data[1]
                p = 2 + (8 if flags & 1 else 0)
                fheap, name_bt = struct.unpack_from("<QQ", data, p)
                if fheap != UNDEF:
                    heap = _FractalHeap(self, fheap)
                    for rec in _BTree2(self, name_bt).records():
                        yield self._link(heap.get(rec[4:4 + heap.id_len]))

    def _link(self, data):
        flags = data[1]
        p = 2
        ltype = 0
        if flags & 0x08:
            ltype = data[p]
            p += 1
        if flags & 0x04:
            p += 8
        if flags & 0x10:
            p += 1
        nb = 1 << (flags & 3)
        n = int.from_bytes(data[p:p + nb], "little")
        p += nb
        name = bytes(data[p:p + n]).decode("utf-8")
        p += n
        if ltype == 0:
            return name, struct.unpack_from("<Q", data, p)[0]
        return name, None

    def _symbol_table(self, btree, heap):
        h = self.at(heap, 32)
        if h[:4] != b"HEAP":
            raise H5Error("bad local heap signature")
        seg_size, _free, seg_addr = struct.unpack_from("<QQQ", h, 8)
        names = self.at(seg_addr, seg_size)

        def name_at(off):
            return bytes(names[off:names.index(b"\0", off)]).decode("utf-8")

        def walk(addr):
            node = self.at(addr, 24)
            if node[:4] != b"TREE" or node[4] != 0:
                raise H5Error("bad group B-tree node")
            level, used = node[5], struct.unpack_from("<H", node, 6)[0]
            body = self.at(addr + 24, (2 * used + 1) * 8)
            children = [struct.unpack_from("<Q", body, 8 + 16 * i)[0] for i in range(used)]
            for c in children:
                if level > 0:
                    yield from walk(c)
                else:
                    snod = self.at(c, 8)
                    if snod[:4] != b"SNOD":
                        raise H5Error("bad symbol table node")
                    count = struct.unpack_from("<H", snod, 6)[0]
                    entries = self.at(c + 8, 40 * count)
                    for i in range(count):
                        off, obj = struct.unpack_from("<QQ", entries, 40 * i)
                        yield name_at(off), obj

        yield from walk(btree)

    def _dense_attributes(self, data):
        flags = data[1]
        p = 2 + (2 if flags & 1 else 0)
        fheap, name_bt = struct.unpack_from("<QQ", data, p)
        if fheap == UNDEF:
            return
        heap = _FractalHeap(self, fheap)
        for rec in _BTree2(self, name_bt).records():
            yield self._attribute(heap.get(rec[0:heap.id_len]))

    # ---- raw data

    def dataset_bytes(self, layout, dt, dims):
        count = int(np.prod(dims)) if dims else (1 if dims == () else 0)
        nbytes = count * dt.size
        out = np.empty(nbytes, np.uint8)
        self.dataset_into(layout, dt, dims, out)
        return out.tobytes()

    def dataset_into(self, layout, dt, dims, out: np.ndarray):
        nbytes = out.nbytes
        if layout["class"] == "compact":
            out[...] = np.frombuffer(layout["data"][:nbytes], np.uint8)
            return
        if layout["class"] == "contiguous":
            if nbytes == 0:
                return
            if layout["addr"] == UNDEF:
                out[...] = 0
                return
            self.f.seek(self.base + layout["addr"])
            got = self.f.readinto(memoryview(out))
            if got != nbytes:
                raise H5Error("dataset data runs past the end of the file")
            return
        self._chunked_into(layout, dt, dims, out)

    def _chunked_into(self, layout, dt, dims, out):
        if any(f not in (1,) for f in layout["filters"]):
            raise H5Error(f"filters {layout['filters']} are not supported (deflate only)")
        chunk = tuple(layout["chunk"])
        esize = dt.size
        full = np.zeros(tuple(dims) if dims else (1,), dtype=np.dtype(f"V{esize}"))
        nd = len(chunk)

        def walk(addr):
            node = self.at(addr, 24)
            if node[:4] != b"TREE" or node[4] != 1:
                raise H5Error("bad chunk B-tree node")
            level, used = node[5], struct.unpack_from("<H", node, 6)[0]
            ksize = 8 + 8 * (nd + 1)
            body = self.at(addr + 24, used * (ksize + 8) + ksize)
            for i in range(used):
                k = i * (ksize + 8)
                csize, _mask = struct.unpack_from("<II", body, k)
                offs = struct.unpack_from(f"<{nd + 1}Q", body, k + 8)
                child = struct.unpack_from("<Q", body, k + ksize)[0]
                if level > 0:
                    walk(child)
                    continue
                raw = self.at(child, csize)
                if layout["filters"]:
                    raw = zlib.decompress(raw)
                block = np.frombuffer(raw, dtype=full.dtype, count=int(np.prod(chunk))).reshape(chunk)
                sl = tuple(slice(o, min(o + c, d)) for o, c, d in zip(offs[:nd], chunk, dims))
                full[sl] = block[tuple(slice(0, s.stop - s.start) for s in sl)]

        if layout["addr"] != UNDEF:
            walk(layout["addr"])
        out[...] = np.frombuffer(full.tobytes(), np.uint8)

    def global_heap_object(self, addr, index):
        if addr not in self._gheaps:
            head = self.at(addr, 16)
            if head[:4] != b"GCOL":
                raise H5Error("bad global heap signature")
            size = struct.unpack_from("<Q", head, 8)[0]
            blob = self.at(addr, size)
            objs = {}
            p = 16
            while p + 16 <= size:
                idx, _refs = struct.unpack_from("<HH", blob, p)
                osize = struct.unpack_from("<Q", blob, p + 8)[0]
                if idx == 0:
                    break
                objs[idx] = bytes(blob[p + 16:p + 16 + osize])
                p += 16 + (osize + 7) // 8 * 8
            self._gheaps[addr] = objs
        return self._gheaps[addr][index]


class _FractalHeap:
    """Format spec III.G: managed objects of a fractal heap (direct blocks under a
    doubling table of indirect blocks) and tiny objects held in the heap ID itself."""

    def __init__(self, r: _Reader, addr):
        self.r = r
        h = r.at(addr, 256)
        if h[:4] != b"FRHP":
            raise H5Error("bad fractal heap signature")
        self.id_len, filt_len = struct.unpack_from("<HH", h, 5)
        self.flags = h[9]
        self.max_managed = struct.unpack_from("<I", h, 10)[0]
        p = 14 + 8 * 12
        self.width = struct.unpack_from("<H", h, p)[0]
        self.start_block, self.max_direct = struct.unpack_from("<QQ", h, p + 2)
        self.max_heap_bits, self.start_rows = struct.unpack_from("<HH", h, p + 18)
        self.root, self.cur_rows = struct.unpack_from("<QH", h, p + 22)
        end = p + 32
        if filt_len:
            raise H5Error("filtered fractal heaps are not supported")
        r._check(h[:end], struct.unpack_from("<I", h, end)[0], "fractal heap header")
        self.off_bytes = (self.max_heap_bits + 7) // 8
        self.len_bytes = _bytes_for(min(self.max_direct, self.max_managed))
        self.addr = addr
        # rows: 0 and 1 hold start_block, each later row double the one before
        self.max_direct_rows = (self.max_direct // self.start_block).bit_length() + 1

    def _row_size(self, row):
        return self.start_block if row <= 1 else self.start_block << (row - 1)

    def get(self, hid: bytes) -> bytes:
        kind = (hid[0] >> 4) & 3
        if kind == 2:  # tiny: length - 1 in the low bits, the data after
            n = (hid[0] & 0x0F) + 1
            return bytes(hid[1:1 + n])
        if kind != 0:
            raise H5Error("huge fractal heap objects are not supported")
        off = int.from_bytes(hid[1:1 + self.off_bytes], "little")
        n = int.from_bytes(hid[1 + self.off_bytes:1 + self.off_bytes + self.len_bytes], "little")
        block, start = self._find(off)
        return self.r.at(block + (off - start), n)

    def _find(self, off):
        """(address, heap offset) of the direct block holding heap offset off."""
        if self.cur_rows == 0:
            return self.root, 0
        return self._find_in(self.root, self.cur_rows, 0, off)

    def _find_in(self, iblock, nrows, base, off):
        head = self.r.at(iblock, 5 + 8 + self.off_bytes)
        if head[:4] != b"FHIB":
            raise H5Error("bad fractal heap indirect block")
        p = 5 + 8 + self.off_bytes
        pos = base
        for row in range(nrows):
            size = self._row_size(row)
            for col in range(self.width):
                entry = p + 8 * (row * self.width + col)
                if pos <= off < pos + size:
                    child = struct.unpack_from("<Q", self.r.at(iblock + entry, 8), 0)[0]
                    if row < self.max_direct_rows:
                        return child, pos
                    return self._find_in(child, self._rows_for(size), pos, off)
                pos += size
        raise H5Error("heap offset outside the heap")

    def _rows_for(self, size):
        # an indirect block covering `size` bytes holds the rows whose total is size
        rows, total = 0, 0
        while total < size:
            total += self._row_size(rows) * self.width
            rows += 1
        return rows


class _BTree2:
    """Format spec III.A.2: the records of a version 2 B-tree, in key order."""

    def __init__(self, r: _Reader, addr):
        self.r = r
        h = r.at(addr, 38)
        if h[:4] != b"BTHD":
            raise H5Error("bad v2 B-tree header")
        self.type = h[5]
        self.node_size, self.rec_size, self.depth = struct.unpack_from("<IHH", h, 6)
        self.root, self.root_n, self.total = struct.unpack_from("<QHQ", h, 16)
        r._check(h[:34], struct.unpack_from("<I", h, 34)[0], "v2 B-tree header")
        # records a node can hold at each depth, for the width of the child-count fields
        leaf_max = (self.node_size - 10) // self.rec_size
        self.max_rec = [leaf_max]
        self.max_total = [leaf_max]
        for d in range(1, self.depth + 1):
            ptr = 8 + _bytes_for(self.max_rec[d - 1]) + (_bytes_for(self.max_total[d - 1]) if d > 1 else 0)
            n = (self.node_size - 10 - ptr) // (self.rec_size + ptr)
            self.max_rec.append(n)
            self.max_total.append((n + 1) * self.max_total[d - 1] + n)

    def records(self):
        if self.root == UNDEF or self.root_n == 0:
            return
        yield from self._node(self.root, self.root_n, self.depth)

    def _node(self, addr, n, depth):
        sig = b"BTLF" if depth == 0 else b"BTIN"
        blob = self.r.at(addr, self.node_size)
        if blob[:4] != sig:
            raise H5Error("bad v2 B-tree node")
        p = 6
        recs = [bytes(blob[p + i * self.rec_size:p + (i + 1) * self.rec_size]) for i in range(n)]
        p += n * self.rec_size
        if depth == 0:
            self.r._check(blob[:p], struct.unpack_from("<I", blob, p)[0], "v2 B-tree leaf")
            yield from recs
            return
        nb = _bytes_for(self.max_rec[depth - 1])
        tb = _bytes_for(self.max_total[depth - 1]) if depth > 1 else 0
        kids = []
        for _ in range(n + 1):
            caddr = struct.unpack_from("<Q", blob, p)[0]
            cn = int.from_bytes(blob[p + 8:p + 8 + nb], "little")
            p += 8 + nb + tb
            kids.append((caddr, cn))
        self.r._check(blob[:p], struct.unpack_from("<I", blob, p)[0], "v2 B-tree internal node")
        for i, (caddr, cn) in enumerate(kids):
            yield from self._node(caddr, cn, depth - 1)
            if i < n:
                yield recs[i]


# ---------------------------------------------------------------------------- writer


def _message(mtype, data, flags=0):
    return struct.pack("<BHB", mtype, len(data), flags) + data


def _object_header(messages: bytes) -> bytes:
    n = len(messages)
    if n < 256:
        flags, size = 0, struct.pack("<B", n)
    elif n < 65536:
        flags, size = 1, struct.pack("<H", n)
    else:
        flags, size = 2, struct.pack("<I", n)
    head = b"OHDR" + bytes([2, flags]) + size + messages
    return head + struct.pack("<I", lookup3(head))


def _array_bytes(a: np.ndarray, dt: np.dtype):
    """A buffer of the array's elements in Fortran order, as dtype dt (no copy when the
    array is already Fortran-contiguous in that dtype)."""
    if a.dtype.kind in "UO":
        a = np.array([str(v).encode("utf-8") for v in a.ravel(order="F")], dtype=dt).reshape(a.shape, order="F")
    a = a.astype(dt, copy=False)
    if a.ndim == 0:
        return a.tobytes()
    flat = np.ascontiguousarray(np.asfortranarray(a).T)  # C-contiguous view of the Fortran bytes
    return memoryview(flat).cast("B")


def _attribute_message(name, value) -> bytes:
    dt, dims, raw = _from_value(value)
    if raw is None:
        raw = bytes(_array_bytes(np.asarray(value), dt))
    tmsg = _encode_datatype(dt)
    smsg = _encode_dataspace(dims)
    nm = name.encode("utf-8") + b"\0"
    return struct.pack("<BBHHHB", 3, 0, len(nm), len(tmsg), len(smsg), 1) + nm + tmsg + smsg + raw


class _Writer:
    """Finishes the output file: the data of datasets still in the file that was read
    is copied over, then every object header is appended and the superblock written."""

    def __init__(self, file: "File"):
        self.file = file

    def _order(self):
        objs, seen = [], set()
        queue = [self.file]
        while queue:
            node = queue.pop(0)
            if id(node) in seen:
                continue
            seen.add(id(node))
            objs.append(node)
            if isinstance(node, Group):
                queue.extend(node._links.values())
        return objs

    def _header_messages(self, node, addr_of):
        msgs = b""
        if isinstance(node, Group):
            msgs += _message(0x02, struct.pack("<BBQQ", 0, 0, UNDEF, UNDEF))
            msgs += _message(0x0A, struct.pack("<BB", 0, 0))
            for lname, child in node._links.items():
                nm = lname.encode("utf-8")
                fl = 0x10 | (0 if len(nm) < 256 else 1)
                ln = struct.pack("<B", len(nm)) if len(nm) < 256 else struct.pack("<H", len(nm))
                msgs += _message(0x06, bytes([1, fl, 1]) + ln + nm + struct.pack("<Q", addr_of(child)))
        else:
            if node._value is not None:
                dt, dims, raw = _from_value(node._value)
                addr, nbytes = node._inline
            else:
                addr, nbytes, dt, dims = node._written
            msgs += _message(0x01, _encode_dataspace(dims))
            msgs += _message(0x03, _encode_datatype(dt), flags=0x01)
            msgs += _message(0x05, struct.pack("<BB", 3, 0x09), flags=0x01)
            c = getattr(node, "_chunked", None)
            if c is not None:
                if c["level"] is not None:
                    # filter pipeline, version 2: deflate (id 1), one client value: the level
                    msgs += _message(0x0B, struct.pack("<BBHHHI", 2, 1, 1, 0, 1, c["level"]), flags=0x01)
                cd = tuple(c["chunk"]) + (np.dtype(dt).itemsize,)
                msgs += _message(0x08, struct.pack(f"<BBBQ{len(cd)}I", 3, 2, len(cd), addr, *cd))
            else:
                msgs += _message(0x08, struct.pack("<BBQQ", 3, 1, addr if nbytes else UNDEF, nbytes))
        for aname, value in node.attrs.items():
            msgs += _message(0x0C, _attribute_message(aname, value))
        return msgs

    def write(self):
        f = self.file
        objs = self._order()
        for o in objs:
            if not isinstance(o, Dataset):
                continue
            if o._value is not None:
                _, _, raw = _from_value(o._value)
                o._inline = f._append_raw(raw)
            elif o._written is None:
                o._written = f._copy_stored(o)
        out = f._out
        out.seek(0, os.SEEK_END)
        start = (out.tell() + 7) // 8 * 8
        out.write(bytes(start - out.tell()))
        index = {id(o): i for i, o in enumerate(objs)}
        sizes = [len(_object_header(self._header_messages(o, lambda c: 0))) for o in objs]
        addrs, p = [], start
        for n in sizes:
            addrs.append(p)
            p += n
        addr_of = lambda o: addrs[index[id(o)]]
        for o, a in zip(objs, addrs):
            assert out.tell() == a
            out.write(_object_header(self._header_messages(o, addr_of)))
        eof = out.tell()
        sb = SIGNATURE + bytes([2, 8, 8, 0]) + struct.pack("<4Q", 0, UNDEF, eof, addrs[0])
        out.seek(0)
        out.write(sb + struct.pack("<I", lookup3(sb)))
        out.flush()


# ---------------------------------------------------------------------------- files


class File(Group):
    """An HDF5 file.  mode "r": read only; "w": create (truncate); "r+": modify an
    existing file; "a" (or Julia's "cw"): modify, creating it if absent.  A dataset's
    data is written when the dataset is created; the file's structure (groups,
    attributes, links) is written when the file is closed or leaves its with-block.
    Until then the new contents live in a temporary file beside the target, which
    replaces the target at close; an exception inside the with-block discards it."""

    def __init__(self, path, mode="r"):
        super().__init__(self, "/")
        self.path = os.fspath(path)
        if mode == "cw":
            mode = "a"
        if mode not in ("r", "w", "r+", "a"):
            raise ValueError(f"mode must be 'r', 'w', 'r+' or 'a', got {mode!r}")
        self.mode = mode
        self._reader = None
        self._out = None
        self._tmp = None
        self._open = True
        if not (mode == "w" or (mode == "a" and not os.path.exists(self.path))):
            self._reader = _Reader(self.path)
            root = self._reader.load(self, self._reader.root_addr, "/", {})
            if not isinstance(root, Group):
                raise H5Error("the root object is not a group")
            self._links = root._links
            self.attrs._items = root.attrs._items
        if mode != "r":
            d = os.path.dirname(os.path.abspath(self.path))
            fd, self._tmp = tempfile.mkstemp(prefix=".h5tmp", dir=d)
            self._out = os.fdopen(fd, "w+b")
            self._out.write(bytes(48))  # the superblock, written at close

    def _writable(self):
        if not self._open:
            raise H5Error("the file is closed")
        if self.mode == "r":
            raise H5Error("the file is open read-only")

    def _append_raw(self, raw):
        out = self._out
        out.seek(0, os.SEEK_END)
        addr = (out.tell() + 7) // 8 * 8
        out.write(bytes(addr - out.tell()))
        out.write(raw)
        return addr, len(raw)

    def _append(self, a: np.ndarray, dt: np.dtype):
        self._writable()
        buf = _array_bytes(a, dt)
        return self._append_raw(buf)

    def _append_chunked(self, a: np.ndarray, dt: np.dtype, chunks, level):
        """Writes the array's chunks (deflated when level is given) and a version 1 B-tree
        of type 1 indexing them; returns (B-tree address, data bytes, chunk entries,
        HDF5-order chunk dims)."""
        self._writable()
        import itertools
        hdf = np.ascontiguousarray(np.asfortranarray(a.astype(dt, copy=False)).T)  # HDF5 (C) order
        cdims = tuple(reversed(chunks))
        entries, total = [], 0
        for offs in itertools.product(*[range(0, n, c) for n, c in zip(hdf.shape, cdims)]):
            sl = tuple(slice(o, min(o + c, n)) for o, c, n in zip(offs, cdims, hdf.shape))
            block = np.zeros(cdims, dtype=hdf.dtype)
            block[tuple(slice(0, q.stop - q.start) for q in sl)] = hdf[sl]
            raw = block.tobytes()
            if level is not None:
                raw = zlib.compress(raw, level)
            addr, n = self._append_raw(raw)
            entries.append((offs, addr, n))
            total += n
        return self._append_chunk_btree(entries, cdims), total, entries, cdims

    def _append_chunk_btree(self, entries, cdims):
        """A version 1 B-tree of chunk records: leaves of up to 64 chunks (2K, K = 32 being
        the format's default), internal levels of up to 64 children, siblings linked, each
        node written at its full size; returns the root's address."""
        nd = len(cdims)
        fan = 64
        ksize = 8 + 8 * (nd + 1)
        node_size = 24 + fan * (ksize + 8) + ksize

        def key(offs, size=0):
            return struct.pack("<II", size, 0) + struct.pack(f"<{nd + 1}Q", *offs, 0)

        # (first offsets, end offsets, [(key bytes, child address)], level) per node
        level = 0
        nodes = [(grp[0][0], tuple(o + c for o, c in zip(grp[-1][0], cdims)),
                  [(key(offs, n), addr) for offs, addr, n in grp], 0)
                 for grp in (entries[i:i + fan] for i in range(0, len(entries), fan))]
        while True:
            first = self._append_raw(b"")[0]
            addrs = [first + i * node_size for i in range(len(nodes))]
            for i, (_, end, kids, lev) in enumerate(nodes):
                left = addrs[i - 1] if i > 0 else UNDEF
                right = addrs[i + 1] if i + 1 < len(nodes) else UNDEF
                body = b"".join(k + struct.pack("<Q", c) for k, c in kids) + key(end)
                head = b"TREE" + struct.pack("<BBHQQ", 1, lev, len(kids), left, right)
                out = self._out
                out.seek(0, os.SEEK_END)
                assert out.tell() == addrs[i]
                out.write(head + body + bytes(node_size - len(head) - len(body)))
            if len(nodes) == 1:
                return addrs[0]
            # the next level: a node per run of up to 64 children, keyed by each child's
            # first chunk, ending at its last child's end
            level += 1
            parents = []
            for j in range(0, len(nodes), fan):
                run = list(zip(nodes[j:j + fan], addrs[j:j + fan]))
                parents.append((run[0][0][0], run[-1][0][1], [(key(child[0]), caddr) for child, caddr in run], level))
            nodes = parents

    def _copy_stored(self, ds: Dataset):
        """Copies a dataset of the file that was read into the output; returns its
        (address, bytes, numpy dtype, HDF5 dims)."""
        reader, dt, dims, layout = ds._stored
        if dt.kind in ("int", "float", "complex") and dt.dtype.byteorder != ">" and layout["class"] == "contiguous":
            count = int(np.prod(dims)) if dims else 1
            left = count * dt.size
            out = self._out
            out.seek(0, os.SEEK_END)
            addr = (out.tell() + 7) // 8 * 8
            out.write(bytes(addr - out.tell()))
            if layout["addr"] == UNDEF:
                out.write(bytes(left))
            else:
                reader.f.seek(reader.base + layout["addr"])
                while left:
                    piece = reader.f.read(min(left, 1 << 26))
                    if not piece:
                        raise H5Error("source dataset truncated")
                    out.write(piece)
                    left -= len(piece)
            return addr, count * dt.size, dt.dtype, dims
        v = ds.read()
        ndt, ndims, raw = _from_value(v)
        if raw is not None:
            addr, n = self._append_raw(raw)
        else:
            addr, n = self._append(np.asarray(v), ndt)
        return addr, n, ndt, ndims

    def _read_output(self, addr, nbytes):
        self._out.flush()
        self._out.seek(addr)
        return self._out.read(nbytes)

    def _discard(self):
        if self._out is not None:
            self._out.close()
            self._out = None
        if self._tmp is not None and os.path.exists(self._tmp):
            os.unlink(self._tmp)
        self._tmp = None
        if self._reader is not None:
            self._reader.close()
            self._reader = None
        self._open = False

    def close(self):
        if not self._open:
            return
        try:
            if self.mode != "r":
                _Writer(self).write()
                self._out.close()
                self._out = None
                if self._reader is not None:
                    self._reader.close()
                    self._reader = None
                os.replace(self._tmp, self.path)
                self._tmp = None
        finally:
            self._discard()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        if exc[0] is not None:
            self._discard()  # an exception inside the block writes nothing
            return False
        self.close()
        return False

    def __del__(self):
        try:
            if getattr(self, "_open", False):
                self._discard()
        except Exception:
            pass


def h5open(path, mode="r") -> File:
    return File(path, mode)
