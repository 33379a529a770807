"""HDF5 checkpoints in the reference's GMPS group layout (gmps.jl:359-383),
written and read by tngpu.h5 without an HDF5 library (none is installed
here or on the GPU machine).

  * Round trips: ragged MPS bond dimensions, an MPO (rank 2), a 100-site
    chain, an unset centre; the reference's error for a group whose type
    attribute is not "MPS".
  * The bytes follow the format's version-0 structures: signature,
    superblock fields, end-of-file address, object-header prefix, local
    heap, B-tree and symbol-table-node signatures, names sorted in the node,
    and each tensor's dimensions reversed (HDF5.jl's column-major
    convention) with its raw bytes in Julia's memory order.
  * The reader follows the structures HDF5.jl files can hold besides those
    the writer emits: a variable-length string attribute in a global heap,
    compact storage, an object-header continuation and a two-level group
    B-tree (a file assembled here from the module's own pieces)."""

import struct

import numpy as np
import pytest

from tngpu import h5


def crand(rng, *shape):
    return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def _mps(rng, dims, d=2):
    return [crand(rng, dims[i], d, dims[i + 1]) for i in range(len(dims) - 1)]


def test_round_trip_ragged_mps(tmp_path):
    rng = np.random.default_rng(1)
    ts = _mps(rng, [1, 2, 4, 7, 3, 1])
    path = str(tmp_path / "psi.h5")
    h5.write_gmps(path, ts, 3, name="ground")
    back, center = h5.read_gmps(path, name="ground")
    assert center == 3 and len(back) == 5
    for a, b in zip(ts, back):
        assert a.shape == b.shape and np.array_equal(a, b)


def test_round_trip_mpo_and_long_chain(tmp_path):
    rng = np.random.default_rng(2)
    mpo = [crand(rng, a, 2, 2, b) for a, b in ((1, 3), (3, 3), (3, 1))]
    p = str(tmp_path / "w.hdf5")
    h5.write_gmps(p, mpo, 0)
    back, center = h5.read_gmps(p)
    assert center == 0 and all(np.array_equal(a, b) for a, b in zip(mpo, back))
    dims = [1] + [4] * 99 + [1]
    ts = _mps(rng, dims)
    p = str(tmp_path / "long.h5")
    h5.write_gmps(p, ts, 100)
    back, center = h5.read_gmps(p)
    assert center == 100 and len(back) == 100
    assert all(np.array_equal(a, b) for a, b in zip(ts, back))


def test_reference_error_for_non_mps_group(tmp_path):
    p = str(tmp_path / "x.h5")
    h5.write_gmps(p, _mps(np.random.default_rng(3), [1, 2, 1]), 1)
    raw = bytearray(open(p, "rb").read())
    i = raw.index(b"MPS\0")  # the type attribute's value
    raw[i:i + 3] = b"QS\0"
    open(p, "wb").write(bytes(raw))
    with pytest.raises(ValueError, match="does not contain MPS data"):
        h5.read_gmps(p)
    with pytest.raises(KeyError):
        h5.read_gmps(p, name="other")
    open(p, "wb").write(b"not hdf5" * 20)
    with pytest.raises(ValueError, match="signature"):
        h5.read_gmps(p)


def test_file_structure(tmp_path):
    rng = np.random.default_rng(4)
    ts = _mps(rng, [1, 2, 3, 1])
    p = str(tmp_path / "s.h5")
    h5.write_gmps(p, ts, 2)
    b = open(p, "rb").read()
    assert b[:8] == b"\x89HDF\r\n\x1a\n"
    assert b[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])  # superblock v0, 8-byte offsets/lengths
    leaf_k, internal_k, flags = struct.unpack_from("<HHI", b, 16)
    assert internal_k == 16 and flags == 0 and 2 * leaf_k >= len(ts) + 2
    base, freespace, eof, driver = struct.unpack_from("<QQQQ", b, 24)
    assert base == 0 and freespace == driver == h5.UNDEF and eof == len(b)
    _, root_hdr, cache, _, btree, heap = struct.unpack_from("<QQIIQQ", b, 56)
    assert cache == 1 and b[btree:btree + 4] == b"TREE" and b[heap:heap + 4] == b"HEAP"
    assert b[root_hdr] == 1  # object header version 1
    nmsgs, size = struct.unpack_from("<H4xI", b, root_hdr + 2)
    assert nmsgs == 1 and size % 8 == 0
    # the group's symbol-table node: names sorted bytewise, one entry each
    r = h5._Reader(b)
    members = r.group(r.group(r.root)["psi"])
    assert sorted(members) == ["MPS[1]", "MPS[2]", "MPS[3]", "center", "length"]
    g_tree, g_heap = struct.unpack_from("<QQ", dict(r.messages(r.group(r.root)["psi"]))[0x11], 0)
    snod = struct.unpack_from("<Q", b, g_tree + 32)[0]  # the B-tree's one child
    assert b[snod:snod + 4] == b"SNOD"
    n = struct.unpack_from("<H", b, snod + 6)[0]
    names = [r.heap_name(g_heap, struct.unpack_from("<Q", b, snod + 8 + 40 * j)[0])
             for j in range(n)]
    assert n == 5 and names == sorted(names, key=str.encode)
    # a tensor dataset: dims reversed, raw bytes in Julia's (column-major) order
    msgs = dict(r.messages(members["MPS[2]"]))
    space = msgs[0x1]
    assert struct.unpack_from("<3Q", space, 8) == (3, 2, 2)
    addr, nbytes = struct.unpack_from("<QQ", msgs[0x8], 2)
    assert b[addr:addr + nbytes] == ts[1].tobytes(order="F")
    assert msgs[0x3][:8] == bytes([0x16, 2, 0, 0]) + struct.pack("<I", 16)  # {r, i} compound
    assert r.attributes(r.group(r.root)["psi"]) == {"type": "MPS", "version": 1}


def _variant_file(tensors, center):
    """A file with the GMPS group laid out the way another writer might:
    the group's attributes in a continuation chunk, "type" a variable-length
    string in a global heap, "length" in compact storage, and the group's
    B-tree two levels deep."""
    buf = bytearray(96)

    def place(blob):
        addr = len(buf)
        buf.extend(h5._pad8(blob))
        return addr

    names = ["length", "center"] + [f"MPS[{i}]" for i in range(1, len(tensors) + 1)]
    grp = h5._Group(names, leaf_k=max(4, -(-len(names) // 2)))
    entries = {}
    # length: compact layout
    hdr = h5._object_header([
        h5._msg(h5._SPACE, h5._space(())), h5._msg(h5._TYPE, h5._dt_int64()),
        h5._msg(h5._LAYOUT, struct.pack("<BBH", 3, 0, 8) + struct.pack("<q", len(tensors)))])
    entries["length"] = h5._entry(grp.offset["length"], place(hdr))
    for nm, dt, dims, raw in [("center", h5._dt_int64(), (), struct.pack("<q", center))] + [
            (f"MPS[{i}]", h5._dt_complex(), tuple(reversed(t.shape)), t.tobytes(order="F"))
            for i, t in enumerate(tensors, start=1)]:
        data = place(raw)
        entries[nm] = h5._entry(grp.offset[nm], place(h5._dataset_header(dt, dims, data, len(raw))))
    heap = len(buf)
    buf.extend(b"\0" * grp.sizes["heap"])
    buf[heap:heap + grp.sizes["heap"]] = grp.heap(heap)
    snod = place(grp.snod(entries))
    leaf = place(grp.tree(snod))
    top = bytearray(grp.tree(leaf))
    top[5] = 1  # level 1: its child is the level-0 node
    top_addr = place(bytes(top))
    # global heap collection holding "MPS"
    obj = struct.pack("<HH4xQ", 1, 1, 3) + h5._pad8(b"MPS")
    gcol = place(b"GCOL" + struct.pack("<B3xQ", 1, 16 + len(obj)) + obj)
    vlen = bytes([0x19, 0x01, 0x00, 0]) + struct.pack("<I", 16) \
        + bytes([0x10, 0, 0, 0]) + struct.pack("<IHH", 1, 0, 8)
    cont = h5._attr_msg("type", vlen, h5._space(()), struct.pack("<IQI", 3, gcol, 1)) \
        + h5._attr_msg("version", h5._dt_int64(), h5._space(()), struct.pack("<q", 1))
    cont_addr = place(cont)
    ghdr = bytearray(h5._object_header([
        h5._msg(h5._STAB, struct.pack("<QQ", top_addr, heap)),
        h5._msg(h5._CONT, struct.pack("<QQ", cont_addr, len(cont)))]))
    struct.pack_into("<H", ghdr, 2, 4)  # four messages: two here, two in the continuation
    g_hdr = place(bytes(ghdr))
    root = h5._Group(["psi"], grp.leaf_k)  # the superblock's leaf K holds for every node
    rheap = len(buf)
    buf.extend(b"\0" * root.sizes["heap"])
    buf[rheap:rheap + root.sizes["heap"]] = root.heap(rheap)
    rsnod = place(root.snod({"psi": h5._entry(root.offset["psi"], g_hdr)}))
    rtree = place(root.tree(rsnod))
    rhdr = place(h5._object_header([h5._msg(h5._STAB, struct.pack("<QQ", rtree, rheap))]))
    sb = h5.SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", grp.leaf_k, 16, 0)
    sb += struct.pack("<QQQQ", 0, h5.UNDEF, len(buf), h5.UNDEF) + h5._entry(0, rhdr, rtree, rheap)
    buf[:96] = sb
    return bytes(buf)


def test_reader_follows_other_writers_structures(tmp_path):
    rng = np.random.default_rng(5)
    ts = _mps(rng, [1, 2, 4, 2, 1])
    p = tmp_path / "variant.h5"
    p.write_bytes(_variant_file(ts, 2))
    back, center = h5.read_gmps(str(p))
    assert center == 2 and all(np.array_equal(a, b) for a, b in zip(ts, back))
    r = h5._Reader(p.read_bytes())
    assert r.attributes(r.group(r.root)["psi"]) == {"type": "MPS", "version": 1}


@pytest.mark.parametrize("ext", [".h5", ".hdf5", ".npz"])
def test_write_mps_read_mps_dispatch(tmp_path, monkeypatch, ext):
    """write_mps/read_mps on a stand-in state (its tensors and centre, as
    a device GMPS or GMPO downloads them) with the upload stubbed: HDF5 for
    .h5/.hdf5 paths, the .npz record otherwise; rank-2 tensors come back as
    a GMPO, rank-1 as a GMPS (gmps.jl:380-382)."""
    from tngpu import mps as M
    rng = np.random.default_rng(6)
    uploads = []
    for cls in (M.GMPS, M.GMPO):
        monkeypatch.setattr(cls, "from_tensors", classmethod(
            lambda c, ts, center=0, ctx=None: uploads.append((c, ts, center)) or c))

    class State:
        def __init__(self, ts, center):
            self._ts, self.center = ts, center

        def tensors(self):
            return self._ts

    for ts, cls in ((_mps(rng, [1, 2, 3, 1]), M.GMPS),
                    ([crand(rng, a, 2, 2, b) for a, b in ((1, 2), (2, 1))], M.GMPO)):
        path = str(tmp_path / ("state" + ext))
        M.write_mps(path, State(ts, 1), name="g")
        assert M.read_mps(path, name="g") is cls
        c, back, center = uploads[-1]
        assert c is cls and center == 1 and all(np.array_equal(a, b) for a, b in zip(ts, back))
    with open(path, "rb") as f:
        assert (f.read(8) == h5.SIGNATURE) == (ext != ".npz")


def test_group_trees_round_trip(tmp_path):
    """write_file/read_file: nested groups (one empty), Int64/Float64
    scalars, real, integer and complex arrays in column-major order,
    group attributes."""
    rng = np.random.default_rng(7)
    real = np.asfortranarray(rng.standard_normal((3, 5)))
    ints = np.arange(12).reshape(3, 4)
    cplx = crand(rng, 2, 3, 4)
    p = str(tmp_path / "tree.h5")
    h5.write_file(p, h5.Group({
        "a": 3, "b": 2.5, "real": real, "ints": ints,
        "sub": h5.Group({"c": cplx, "deeper": h5.Group({"z": 1j}), "empty": h5.Group()},
                        attrs={"note": "x", "n": 7, "w": 0.25})}))
    got = h5.read_file(p)
    assert got["a"] == 3 and got["b"] == 2.5
    assert np.array_equal(got["real"], real) and np.array_equal(got["ints"], ints)
    assert np.array_equal(got["sub"]["c"], cplx) and got["sub"]["deeper"]["z"] == 1j
    assert got["sub"]["empty"] == {}
    r = h5._Reader(open(p, "rb").read())
    assert r.attributes(r.group(r.root)["sub"]) == {"note": "x", "n": 7, "w": 0.25}
    with pytest.raises(TypeError):
        h5.write_file(p, h5.Group({"flag": True}))


def test_qjmc_activity_saves_time_and_jumps(tmp_path):
    """QJMCActivity(save=true, savefile) (qjmc.jl:275-284) rewrites the file
    with "time" and "jumps" at every measurement."""
    import tngpu as tn
    p = str(tmp_path / "activity.h5")
    obs = tn.QJMCActivity(True, p)
    obs.measure(0.5, None, [3], [0.2])
    assert h5.read_file(p) == {"time": 0.5, "jumps": 1}
    obs.measure(1.25, None, [3, 1, 2], [0.2, 0.9, 1.1])
    got = h5.read_file(p)
    assert got == {"time": 1.25, "jumps": 3} and isinstance(got["jumps"], np.integer)
    quiet = tn.QJMCActivity()
    quiet.measure(1.0, None, [], [])
    assert (quiet.time, quiet.jumps) == (1.0, 0)
