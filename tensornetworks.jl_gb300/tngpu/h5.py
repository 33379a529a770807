"""HDF5 files in HDF5.jl's layout: GMPS checkpoints (gmps.jl:359-383) and
the record of QJMCActivity (qjmc.jl:275-284).

The reference saves a GMPS with HDF5.jl as one group holding:

- attributes ``type`` = "MPS" and ``version`` = 1;
- scalar Int64 datasets ``length`` and ``center``;
- the site tensors as datasets ``MPS[1]`` ... ``MPS[N]``.

Tensors are ComplexF64 arrays, [Dl, d, Dr] for an MPS and [Dl, d, d, Dr]
for an MPO.  HDF5.jl stores a column-major array with its dimensions
reversed, so the raw bytes keep Julia's memory order.  A complex number is
the compound {r: f64, i: f64}.

No HDF5 library is a dependency here, so this module writes and reads that
layout itself, in the HDF5 file format's original structures:

- a version-0 superblock;
- version-1 object headers;
- groups as symbol tables (a local heap of names, a version-1 group B-tree,
  and symbol-table nodes);
- contiguous datasets.

These are the structures the HDF5 library writes by default.  The reader
also follows object-header continuation messages, compact storage,
multi-level group B-trees, and variable-length string attributes (the
global heap), so that files from HDF5.jl in its default file format can be
read too.
"""

import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
FREE_NULL = 1  # end of a local heap's free list
BTREE_K = 16  # group B-tree nodes hold up to 2K children

# object header message types
_NIL, _SPACE, _TYPE, _FILL, _LAYOUT, _CONT, _ATTR, _STAB = 0x0, 0x1, 0x3, 0x5, 0x8, 0x10, 0xC, 0x11


def _pad8(b):
    return b + b"\0" * (-len(b) % 8)


# ---- datatype and dataspace descriptions ---------------------------------------
def _dt_int64():
    # fixed-point, version 1, little-endian, signed; offset 0, precision 64
    return bytes([0x10, 0x08, 0, 0]) + struct.pack("<IHH", 8, 0, 64)


def _dt_f64():
    # floating-point, version 1, little-endian, implied leading mantissa bit,
    # sign at bit 63; exponent bits 52-62 (bias 1023), mantissa bits 0-51
    return bytes([0x11, 0x20, 63, 0]) + struct.pack("<IHHBBBBI", 8, 0, 64, 52, 11, 0, 52, 1023)


def _dt_complex():
    # compound, version 1, two members "r" and "i" (HDF5.jl's ComplexF64)
    body = b""
    for name, off in ((b"r", 0), (b"i", 8)):
        body += _pad8(name + b"\0") + struct.pack("<IB3xI4x4I", off, 0, 0, 0, 0, 0, 0) + _dt_f64()
    return bytes([0x16, 2, 0, 0]) + struct.pack("<I", 16) + body


def _dt_string(n):
    # string, version 1, null-terminated ASCII, n bytes including the null
    return bytes([0x13, 0x00, 0, 0]) + struct.pack("<I", n)


def _space(dims):
    """Simple dataspace, version 1; dims in HDF5's (C) order, () = scalar."""
    return struct.pack("<BBBB4x", 1, len(dims), 0, 0) + b"".join(struct.pack("<Q", d) for d in dims)


# ---- object headers ----------------------------------------------------------------
def _msg(mtype, data):
    data = _pad8(data)
    return struct.pack("<HHB3x", mtype, len(data), 0) + data


def _object_header(msgs):
    body = b"".join(msgs)
    return struct.pack("<BBHII4x", 1, 0, len(msgs), 1, len(body)) + body


def _attr_msg(name, dtype, space, data):
    nm = name.encode() + b"\0"
    return _msg(_ATTR, struct.pack("<BBHHH", 1, 0, len(nm), len(dtype), len(space))
                + _pad8(nm) + _pad8(dtype) + _pad8(space) + data)


def _dataset_header(dtype, dims, data_addr, nbytes):
    return _object_header([
        _msg(_SPACE, _space(dims)),
        _msg(_TYPE, dtype),
        _msg(_FILL, struct.pack("<BBBB", 2, 2, 2, 0)),  # version 2, late, if set, undefined
        _msg(_LAYOUT, struct.pack("<BBQQ", 3, 1, data_addr, nbytes)),  # version 3, contiguous
    ])


def _entry(name_off, ohdr, btree=None, heap=None):
    """Symbol-table entry; groups carry their B-tree and heap addresses."""
    if btree is None:
        return struct.pack("<QQII16x", name_off, ohdr, 0, 0)
    return struct.pack("<QQIIQQ", name_off, ohdr, 1, 0, btree, heap)


class _Group:
    """The symbol-table structures of one group: local heap, B-tree, node."""

    def __init__(self, names, leaf_k):
        self.names = sorted(names, key=lambda s: s.encode())
        heap = bytearray(8)  # offset 0: the empty name, key 0 of the B-tree
        self.offset = {}
        for n in self.names:
            self.offset[n] = len(heap)
            heap += _pad8(n.encode() + b"\0")
        self.heap_data = bytes(heap)
        self.leaf_k = leaf_k
        self.sizes = {"heap": 32 + len(self.heap_data), "snod": 8 + 2 * leaf_k * 40,
                      "tree": 24 + 2 * BTREE_K * 8 + (2 * BTREE_K + 1) * 8}

    def heap(self, addr):
        return (b"HEAP" + struct.pack("<B3xQQQ", 0, len(self.heap_data), FREE_NULL, addr + 32)
                + self.heap_data)

    def snod(self, entries):
        out = b"SNOD" + struct.pack("<BBH", 1, 0, len(self.names))
        out += b"".join(entries[n] for n in self.names)
        return out + b"\0" * (self.sizes["snod"] - len(out))

    def tree(self, snod_addr):
        """A leaf B-tree node over the one symbol-table node, or with no
        children for an empty group."""
        used = 0 if snod_addr is None else 1
        out = b"TREE" + struct.pack("<BBHQQ", 0, 0, used, UNDEF, UNDEF) + struct.pack("<Q", 0)
        if used:
            out += struct.pack("<QQ", snod_addr, self.offset[self.names[-1]])
        return out + b"\0" * (self.sizes["tree"] - len(out))


class Group:
    """A group to write: ``members`` maps names to sub-Groups or dataset
    values, ``attrs`` names to attribute values.  Values follow HDF5.jl's
    conventions: str (fixed-length string), int (Int64), float (Float64),
    and numpy arrays or scalars of integers, floats or complex numbers
    (column-major arrays stored with their dimensions reversed)."""

    def __init__(self, members=None, attrs=None):
        self.members = dict(members or {})
        self.attrs = dict(attrs or {})


def _encode(v):
    """(datatype, HDF5 dims, raw bytes) of a value."""
    if isinstance(v, str):
        b = v.encode() + b"\0"
        return _dt_string(len(b)), (), b
    if isinstance(v, (bool, np.bool_)):
        raise TypeError("booleans have no HDF5.jl counterpart here")
    if isinstance(v, (int, np.integer)):
        return _dt_int64(), (), struct.pack("<q", int(v))
    if isinstance(v, (float, np.floating)):
        return _dt_f64(), (), struct.pack("<d", float(v))
    a = np.asarray(v)
    if np.iscomplexobj(a):
        a, dt = a.astype(np.complex128), _dt_complex()
    elif a.dtype.kind == "f":
        a, dt = a.astype(np.float64), _dt_f64()
    elif a.dtype.kind in "iu":
        a, dt = a.astype(np.int64), _dt_int64()
    else:
        raise TypeError(f"cannot store values of dtype {a.dtype}")
    if a.ndim == 0:
        return dt, (), a.tobytes()
    return dt, tuple(reversed(a.shape)), np.asfortranarray(a).tobytes(order="F")


def write_file(path, root):
    """Write the Group ``root`` and everything under it as a new HDF5 file."""
    def most(g):
        subs = [most(m) for m in g.members.values() if isinstance(m, Group)]
        return max([len(g.members)] + subs)

    leaf_k = max(4, -(-most(root) // 2))  # each group's entries fit one node
    eof = 96  # the superblock
    writes = []

    def reserve(size):
        nonlocal eof
        addr = eof
        eof += -(-size // 8) * 8
        return addr

    def place(g):
        """Lay out g's members, then g; (object header, B-tree, heap)."""
        st = _Group(list(g.members), leaf_k)
        entries = {}
        for name, m in g.members.items():
            if isinstance(m, Group):
                entries[name] = _entry(st.offset[name], *place(m))
                continue
            dt, dims, raw = _encode(m)
            hdr = reserve(len(_dataset_header(dt, dims, 0, len(raw))))
            data = reserve(len(raw))
            writes.append((hdr, _dataset_header(dt, dims, data, len(raw))))
            writes.append((data, raw))
            entries[name] = _entry(st.offset[name], hdr)
        heap = reserve(st.sizes["heap"])
        tree = reserve(st.sizes["tree"])
        writes.append((heap, st.heap(heap)))
        if entries:
            snod = reserve(st.sizes["snod"])
            writes.append((snod, st.snod(entries)))
            writes.append((tree, st.tree(snod)))
        else:
            writes.append((tree, st.tree(None)))
        attrs = []
        for k, v in g.attrs.items():
            dt, dims, raw = _encode(v)
            attrs.append(_attr_msg(k, dt, _space(dims), raw))
        hdr_bytes = _object_header([_msg(_STAB, struct.pack("<QQ", tree, heap))] + attrs)
        hdr = reserve(len(hdr_bytes))
        writes.append((hdr, hdr_bytes))
        return hdr, tree, heap

    r_hdr, r_tree, r_heap = place(root)
    buf = bytearray(eof)
    for addr, b in writes:
        buf[addr:addr + len(b)] = b
    sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", leaf_k, BTREE_K, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF) + _entry(0, r_hdr, r_tree, r_heap)
    buf[:len(sb)] = sb
    with open(path, "wb") as f:
        f.write(bytes(buf))


def write_gmps(path, tensors, center, name="psi"):
    """Write one GMPS group ``name`` (gmps.jl:359-370) as a new HDF5 file.
    ``tensors``: the site arrays, [Dl, d, Dr] or [Dl, d, d, Dr] complex."""
    if len(tensors) == 0:
        raise ValueError("an MPS needs at least one site")
    members = {"length": len(tensors), "center": int(center)}
    for i, t in enumerate(tensors, start=1):
        members[f"MPS[{i}]"] = np.asarray(t, dtype=np.complex128)
    write_file(path, Group({name: Group(members, {"type": "MPS", "version": 1})}))


# ---- reading -------------------------------------------------------------------------
class _Reader:
    def __init__(self, data):
        self.b = data
        if data[:8] != SIGNATURE:
            raise ValueError("not an HDF5 file (signature)")
        ver = data[8]
        if ver not in (0, 1):
            raise NotImplementedError(f"HDF5 superblock version {ver} (only 0 and 1 are read)")
        if data[13] != 8 or data[14] != 8:
            raise NotImplementedError("HDF5 offsets and lengths other than 8 bytes")
        p = 24 + (4 if ver == 1 else 0)
        self.base = self.u64(p)
        self.root = self.u64(p + 32 + 8)  # root entry: object header address

    def u64(self, p):
        return struct.unpack_from("<Q", self.b, p)[0]

    def at(self, addr):
        return self.base + addr

    def messages(self, addr):
        """(type, data) of every message of the object header at addr."""
        p = self.at(addr)
        if self.b[p] != 1:
            raise NotImplementedError("object header version other than 1")
        nmsgs, size = struct.unpack_from("<H4xI", self.b, p + 2)
        chunks, out = [(p + 16, size)], []
        while chunks and len(out) < nmsgs:
            q, size = chunks.pop(0)
            end = q + size
            while q + 8 <= end and len(out) < nmsgs:
                mtype, msize = struct.unpack_from("<HH", self.b, q)
                data = self.b[q + 8:q + 8 + msize]
                out.append((mtype, data))
                if mtype == _CONT:
                    caddr, clen = struct.unpack_from("<QQ", data, 0)
                    chunks.append((self.at(caddr), clen))
                q += 8 + msize
        return out

    def heap_name(self, heap, off):
        if self.b[self.at(heap):self.at(heap) + 4] != b"HEAP":
            raise ValueError("corrupt local heap")
        data = self.at(self.u64(self.at(heap) + 24))
        end = self.b.index(b"\0", data + off)
        return self.b[data + off:end].decode()

    def group(self, addr):
        """{name: object header address} of the group whose header is at addr."""
        stab = [d for t, d in self.messages(addr) if t == _STAB]
        if not stab:
            raise NotImplementedError("group without a symbol table (new-style links)")
        tree, heap = struct.unpack_from("<QQ", stab[0], 0)
        out = {}
        self._walk(tree, heap, out)
        return out

    def _walk(self, node, heap, out):
        p = self.at(node)
        if self.b[p:p + 4] != b"TREE" or self.b[p + 4] != 0:
            raise ValueError("corrupt group B-tree")
        level, used = self.b[p + 5], struct.unpack_from("<H", self.b, p + 6)[0]
        for i in range(used):
            child = self.u64(p + 24 + 8 + 16 * i)
            if level > 0:
                self._walk(child, heap, out)
                continue
            s = self.at(child)
            if self.b[s:s + 4] != b"SNOD":
                raise ValueError("corrupt symbol-table node")
            for j in range(struct.unpack_from("<H", self.b, s + 6)[0]):
                e = s + 8 + 40 * j
                out[self.heap_name(heap, self.u64(e))] = self.u64(e + 8)

    def _vlen_string(self, raw):
        n, coll, idx = struct.unpack_from("<IQI", raw, 0)
        p = self.at(coll)
        if self.b[p:p + 4] != b"GCOL":
            raise ValueError("corrupt global heap")
        q, end = p + 16, p + self.u64(p + 8)
        while q + 16 <= end:
            oidx, _, osize = struct.unpack_from("<HH4xQ", self.b, q)
            if oidx == idx:
                return self.b[q + 16:q + 16 + n].decode()
            if oidx == 0:
                break
            q += 16 + -(-osize // 8) * 8
        raise ValueError("global heap object not found")

    def _decode(self, dtype, dims, raw):
        cls, size = dtype[0] & 0x0F, struct.unpack_from("<I", dtype, 4)[0]
        count = int(np.prod(dims)) if dims else 1
        if cls == 0:  # fixed-point
            signed, big = bool(dtype[1] & 0x08), bool(dtype[1] & 0x01)
            kind = ("i" if signed else "u") + str(size)
            arr = np.frombuffer(raw, dtype=(">" if big else "<") + kind, count=count)
        elif cls == 1:  # floating-point
            arr = np.frombuffer(raw, dtype=(">f" if dtype[1] & 0x01 else "<f") + str(size),
                                count=count)
        elif cls == 6 and size == 16:  # {r, i} complex of two f64
            arr = np.frombuffer(raw, dtype="<c16", count=count)
        elif cls == 3:  # fixed-length string
            return raw[:size].split(b"\0")[0].decode()
        elif cls == 9 and (dtype[1] & 0x0F) == 1:  # variable-length string
            return self._vlen_string(raw)
        else:
            raise NotImplementedError(f"HDF5 datatype class {cls} of size {size}")
        if not dims:
            return arr[0]
        return np.array(arr.reshape(tuple(reversed(dims)), order="F"))

    @staticmethod
    def _dims(space):
        ver, rank = space[0], space[1]
        off = 8 if ver == 1 else 4
        if ver >= 2 and space[3] == 0:
            return ()
        return tuple(struct.unpack_from("<Q", space, off + 8 * k)[0] for k in range(rank))

    def attributes(self, addr):
        out = {}
        for t, d in self.messages(addr):
            if t != _ATTR:
                continue
            ver = d[0]
            nlen, tlen, slen = struct.unpack_from("<HHH", d, 2)
            p = 8 + (1 if ver == 3 else 0)
            pad = (lambda n: -(-n // 8) * 8) if ver == 1 else (lambda n: n)
            name = d[p:p + nlen].split(b"\0")[0].decode()
            p += pad(nlen)
            dtype = d[p:p + tlen]
            p += pad(tlen)
            dims = self._dims(d[p:p + slen])
            p += pad(slen)
            out[name] = self._decode(dtype, dims, d[p:])
        return out

    def dataset(self, addr):
        dtype = dims = raw = None
        for t, d in self.messages(addr):
            if t == _SPACE:
                dims = self._dims(d)
            elif t == _TYPE:
                dtype = d
            elif t == _LAYOUT:
                if d[0] != 3:
                    raise NotImplementedError("data layout message version other than 3")
                if d[1] == 1:
                    a, n = struct.unpack_from("<QQ", d, 2)
                    raw = self.b[self.at(a):self.at(a) + n]
                elif d[1] == 0:
                    n = struct.unpack_from("<H", d, 2)[0]
                    raw = d[4:4 + n]
                else:
                    raise NotImplementedError("chunked datasets")
        return self._decode(dtype, dims, raw)


def read_gmps(path, name="psi"):
    """(tensors, center) of the GMPS group ``name`` of an HDF5 file
    (gmps.jl:372-383), with the reference's check of the type attribute."""
    with open(path, "rb") as f:
        r = _Reader(f.read())
    root = r.group(r.root)
    if name not in root:
        raise KeyError(f"no group {name!r} in {path}")
    if r.attributes(root[name]).get("type") != "MPS":
        raise ValueError("HDF5 group of file does not contain MPS data.")
    members = r.group(root[name])
    N = int(r.dataset(members["length"]))
    center = int(r.dataset(members["center"]))
    return [r.dataset(members[f"MPS[{i}]"]) for i in range(1, N + 1)], center


def read_file(path):
    """Every dataset of an HDF5 file, as nested dicts by group."""
    with open(path, "rb") as f:
        r = _Reader(f.read())

    def walk(addr):
        out = {}
        for name, a in r.group(addr).items():
            if any(t == _STAB for t, _ in r.messages(a)):
                out[name] = walk(a)
            else:
                out[name] = r.dataset(a)
        return out

    return walk(r.root)
