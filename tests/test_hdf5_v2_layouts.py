"""The reader on the newer on-disk structures (what libhdf5 writes with
libver="latest"): superblock version 2, version-2 object headers with their
checksums and a continuation block, compact link messages, dataspace
version 2, fill value version 3, layout version 4 (contiguous, and chunked
with the single-chunk, implicit and fixed-array indexes), filter pipeline
version 2, attribute version 3.  No file of this kind exists here, so a
test-only encoder builds them from the published format specification; the
checks are that every structure parses and every value comes back."""

from __future__ import annotations

import struct
import zlib

import numpy as np
import pytest

from ptylab_gb300.io import hdf5

U = hdf5.UNDEF


def ohdr(messages, continuation=None):
    """A version-2 object header (4-byte chunk size field)."""
    body = b"".join(struct.pack("<BHB", t, len(d), f) + d for t, d, f in messages)
    if continuation is not None:
        body += struct.pack("<BHB", hdf5.MSG_CONTINUATION, 16, 0) + struct.pack("<QQ", *continuation)
    head = b"OHDR" + struct.pack("<BBI", 2, 2, len(body))
    blob = head + body
    return blob + struct.pack("<I", hdf5.lookup3(blob))


def ochk(messages):
    body = b"OCHK" + b"".join(struct.pack("<BHB", t, len(d), f) + d for t, d, f in messages)
    return body + struct.pack("<I", hdf5.lookup3(body))


def dataspace2(shape):
    return struct.pack("<BBBB", 2, len(shape), 0, 1 if shape else 0) + b"".join(struct.pack("<Q", n) for n in shape)


def link(name, addr):
    nb = name.encode()
    return struct.pack("<BBB", 1, 0, len(nb)) + nb + struct.pack("<Q", addr)


FILL3 = struct.pack("<BB", 3, 0x0A)


class Builder:
    def __init__(self):
        self.buf = bytearray(48)  # superblock v2, written last

    def put(self, blob, align=8):
        self.buf += b"\0" * ((-len(self.buf)) % align)
        a = len(self.buf)
        self.buf += blob
        return a

    def reserve(self, n):
        return self.put(b"\0" * n)

    def finish(self, root):
        sb = hdf5.SIGNATURE + struct.pack("<BBBB", 2, 8, 8, 0) + struct.pack("<QQQQ", 0, U, len(self.buf), root)
        sb += struct.pack("<I", hdf5.lookup3(sb))
        self.buf[:48] = sb
        return bytes(self.buf)


def dataset(b, arr, layout, extra=()):
    msgs = [(hdf5.MSG_DATASPACE, dataspace2(arr.shape), 0),
            (hdf5.MSG_DATATYPE, hdf5._encode_datatype(arr.dtype), 1),
            (hdf5.MSG_FILL, FILL3, 1)]
    msgs += list(extra)
    msgs.append((hdf5.MSG_LAYOUT, layout, 0))
    return b.put(ohdr(msgs))


@pytest.fixture(scope="module")
def v2file(tmp_path_factory):
    rng = np.random.default_rng(11)
    want = {}
    b = Builder()
    # contiguous
    a = rng.standard_normal((5, 7)).astype(np.float32)
    addr = b.put(a.tobytes())
    objs = {"contig": dataset(b, a, struct.pack("<BBQQ", 4, 1, addr, a.nbytes))}
    want["contig"] = a
    # single chunk, deflate through a version-2 pipeline
    c = (rng.standard_normal((6, 4)) + 1j * rng.standard_normal((6, 4))).astype(np.complex64)
    raw = zlib.compress(c.tobytes(), 6)
    caddr = b.put(raw)
    lay = struct.pack("<BBBBB", 4, 2, 0x02, 3, 4) + struct.pack("<III", 6, 4, 8) + struct.pack("<B", 1)
    lay += struct.pack("<QI", len(raw), 0) + struct.pack("<Q", caddr)
    pipe = struct.pack("<BB", 2, 1) + struct.pack("<HHH", hdf5.FILTER_DEFLATE, 1, 1) + struct.pack("<I", 6)
    objs["single_chunk_gzip"] = dataset(b, c, lay, [(hdf5.MSG_PIPELINE, pipe, 0)])
    want["single_chunk_gzip"] = c
    # implicit index: unfiltered chunks in row-major order, edge chunks full size
    m = np.arange(7 * 10, dtype=np.int32).reshape(7, 10)
    chunk = (3, 4)
    grid = (3, 3)
    blocks = b""
    for i in range(grid[0]):
        for j in range(grid[1]):
            blk = np.zeros(chunk, np.int32)
            part = m[i * 3:(i + 1) * 3, j * 4:(j + 1) * 4]
            blk[: part.shape[0], : part.shape[1]] = part
            blocks += blk.tobytes()
    iaddr = b.put(blocks)
    lay = struct.pack("<BBBBB", 4, 2, 0, 3, 4) + struct.pack("<III", 3, 4, 4) + struct.pack("<B", 2) + struct.pack("<Q", iaddr)
    objs["implicit"] = dataset(b, m, lay)
    want["implicit"] = m
    # fixed-array index, unpaged, unfiltered chunks stored out of order
    f = rng.standard_normal((4, 6)).astype(np.float64)
    order = [(1, 1), (0, 0), (1, 0), (0, 1)]
    where = {}
    for i, j in order:
        where[(i, j)] = b.put(np.ascontiguousarray(f[i * 2:(i + 1) * 2, j * 3:(j + 1) * 3]).tobytes())
    elems = b"".join(struct.pack("<Q", where[(i, j)]) for i in range(2) for j in range(2))
    fahd_addr = len(b.buf) + ((-len(b.buf)) % 8)
    fahd_len = 4 + 4 + 8 + 8 + 4
    fadb = b"FADB" + struct.pack("<BBQ", 0, 0, fahd_addr) + elems
    fadb += struct.pack("<I", hdf5.lookup3(fadb))
    fahd = b"FAHD" + struct.pack("<BBBB", 0, 0, 8, 10) + struct.pack("<Q", 4)
    fadb_addr = fahd_addr + fahd_len
    fahd += struct.pack("<Q", fadb_addr)
    fahd += struct.pack("<I", hdf5.lookup3(fahd))
    assert b.put(fahd) == fahd_addr and len(fahd) == fahd_len
    assert b.put(fadb, align=1) == fadb_addr
    lay = struct.pack("<BBBBB", 4, 2, 0, 3, 4) + struct.pack("<III", 2, 3, 8) + struct.pack("<BB", 3, 10)
    lay += struct.pack("<Q", fahd_addr)
    objs["fixed_array"] = dataset(b, f, lay)
    want["fixed_array"] = f
    # a scalar with a version-3 attribute
    s = np.array(2.5)
    saddr = b.put(s.tobytes())
    name = b"units"
    tdt = struct.pack("<B3sI", 0x13, (0).to_bytes(3, "little"), 6)
    sds = dataspace2(())
    attr = struct.pack("<BBHHHB", 3, 0, len(name), len(tdt), len(sds), 0) + name + tdt + sds + b"metres"
    objs["scalar"] = dataset(b, s, struct.pack("<BBQQ", 4, 1, saddr, 8), [(hdf5.MSG_ATTRIBUTE, attr, 0)])
    want["scalar"] = s
    # a subgroup with one link, and the root group: links split across a continuation block
    sub_ds = dataset(b, a, struct.pack("<BBQQ", 4, 1, addr, a.nbytes))
    li = struct.pack("<BBQQ", 0, 0, U, U)
    gi = struct.pack("<BB", 0, 0)
    sub = b.put(ohdr([(hdf5.MSG_LINK_INFO, li, 0), (hdf5.MSG_GROUP_INFO, gi, 0), (hdf5.MSG_LINK, link("inner", sub_ds), 0)]))
    names = sorted(objs)
    first, rest = names[:2], names[2:]
    cont = ochk([(hdf5.MSG_LINK, link(n, objs[n]), 0) for n in rest] + [(hdf5.MSG_LINK, link("group", sub), 0)])
    caddr = b.put(cont)
    root = b.put(ohdr([(hdf5.MSG_LINK_INFO, li, 0), (hdf5.MSG_GROUP_INFO, gi, 0)]
                      + [(hdf5.MSG_LINK, link(n, objs[n]), 0) for n in first], continuation=(caddr, len(cont))))
    path = tmp_path_factory.mktemp("v2") / "latest.h5"
    path.write_bytes(b.finish(root))
    return path, want


def test_v2_structures_read_back(v2file):
    path, want = v2file
    with hdf5.File(path) as f:
        assert f.keys() == sorted(list(want) + ["group"])
        for k, v in want.items():
            got = f[k][()]
            assert got.shape == v.shape and got.dtype == v.dtype, k
            np.testing.assert_array_equal(got, v, err_msg=k)
        assert f["scalar"].attrs == {"units": b"metres"}
        np.testing.assert_array_equal(f["group/inner"][()], want["contig"])
        assert "group/inner" in f and "group/missing" not in f


def test_v2_checksums_are_checked(v2file, tmp_path):
    path, _ = v2file
    buf = bytearray(path.read_bytes())
    bad = tmp_path / "bad_superblock.h5"
    buf2 = bytearray(buf)
    buf2[12] ^= 0xFF  # base address byte inside the checksummed superblock
    bad.write_bytes(bytes(buf2))
    with pytest.raises(hdf5.HDF5FormatError):
        hdf5.File(bad)
    i = buf.find(b"OCHK")
    buf3 = bytearray(buf)
    buf3[i + 6] ^= 0x01  # inside the continuation block's first message
    bad2 = tmp_path / "bad_continuation.h5"
    bad2.write_bytes(bytes(buf3))
    with pytest.raises(hdf5.HDF5FormatError):
        hdf5.File(bad2)


def vlen_type(kind, base, charset=0):
    """Datatype message of a variable-length string (kind 1) or sequence (0)."""
    bits = kind | (charset << 8)
    return struct.pack("<B3sI", 0x19, bits.to_bytes(3, "little"), 16) + base


def global_heap(objects):
    """A global heap collection holding ``objects`` (index 1, 2, ...)."""
    body = b""
    for i, data in enumerate(objects, start=1):
        body += struct.pack("<HHIQ", i, 1, 0, len(data)) + data + b"\0" * ((-len(data)) % 8)
    body += struct.pack("<HHIQ", 0, 0, 0, 0)  # free space
    size = 16 + len(body)
    return b"GCOL" + struct.pack("<B3xQ", 1, size) + body


def test_variable_length_strings_and_sequences(tmp_path):
    """h5py writes Python strings as variable-length strings in a global heap;
    sequences of int32 the same way."""
    b = Builder()
    texts = ["LED array, 4 mm pitch", "", "ünïcode"]
    seqs = [np.arange(3, dtype=np.int32), np.array([7], dtype=np.int32)]
    heap_objs = [texts[0].encode(), texts[2].encode("utf-8"), seqs[0].tobytes(), seqs[1].tobytes(),
                 b"metres"]
    gaddr = b.put(global_heap(heap_objs))
    u8 = struct.pack("<B3sIHH", 0x10, b"\0\0\0", 1, 0, 8)
    i32 = hdf5._encode_datatype(np.dtype("<i4"))
    # 1-D string dataset: (length, collection, index); the empty string has length 0
    recs = struct.pack("<IQI", len(heap_objs[0]), gaddr, 1) + struct.pack("<IQI", 0, 0, 0) + \
        struct.pack("<IQI", len(heap_objs[1]), gaddr, 2)
    saddr = b.put(recs)
    tstr = vlen_type(1, u8, charset=1)
    sattr_name = b"units"
    sds = dataspace2(())
    attr = struct.pack("<BBHHHB", 3, 0, len(sattr_name), len(tstr), len(sds), 1) + sattr_name + tstr + sds + \
        struct.pack("<IQI", 6, gaddr, 5)
    d1 = b.put(ohdr([(hdf5.MSG_DATASPACE, dataspace2((3,)), 0), (hdf5.MSG_DATATYPE, tstr, 1),
                     (hdf5.MSG_ATTRIBUTE, attr, 0),
                     (hdf5.MSG_LAYOUT, struct.pack("<BBQQ", 4, 1, saddr, len(recs)), 0)]))
    recs2 = struct.pack("<IQI", 3, gaddr, 3) + struct.pack("<IQI", 1, gaddr, 4)
    qaddr = b.put(recs2)
    d2 = b.put(ohdr([(hdf5.MSG_DATASPACE, dataspace2((2,)), 0), (hdf5.MSG_DATATYPE, vlen_type(0, i32), 1),
                     (hdf5.MSG_LAYOUT, struct.pack("<BBQQ", 4, 1, qaddr, len(recs2)), 0)]))
    # a scalar string in compact storage
    rec3 = struct.pack("<IQI", len(heap_objs[0]), gaddr, 1)
    d3 = b.put(ohdr([(hdf5.MSG_DATASPACE, dataspace2(()), 0), (hdf5.MSG_DATATYPE, tstr, 1),
                     (hdf5.MSG_LAYOUT, struct.pack("<BBH", 4, 0, len(rec3)) + rec3, 0)]))
    li = struct.pack("<BBQQ", 0, 0, U, U)
    root = b.put(ohdr([(hdf5.MSG_LINK_INFO, li, 0), (hdf5.MSG_LINK, link("comment", d1), 0),
                       (hdf5.MSG_LINK, link("runs", d2), 0), (hdf5.MSG_LINK, link("title", d3), 0)]))
    path = tmp_path / "vlen.h5"
    path.write_bytes(b.finish(root))
    with hdf5.File(path) as f:
        got = f["comment"][()]
        assert got.dtype == object and list(got) == texts
        assert f["comment"].dtype == np.dtype(object)
        assert f["comment"].attrs == {"units": "metres"}
        runs = f["runs"][()]
        assert len(runs) == 2 and all(np.array_equal(r, s) for r, s in zip(runs, seqs))
        assert f["title"][()] == texts[0]


def dense_group(b, links, root_indirect=False):
    """A group whose links live in a fractal heap (dense storage) with a
    one-leaf version-2 name index; returns the group's header address."""
    width, start, max_direct, heap_bits = 4, 512, 65536, 32
    off_bytes, len_bytes = 4, 2  # id = type byte + offset + length = 7 bytes
    msgs = [link(n, a) for n, a in links]
    # objects packed after a 32-byte block header area
    hdr_room = 32
    placed, off = [], hdr_room
    for m in msgs:
        placed.append((off, len(m)))
        off += len(m)
    assert off <= start
    block = bytearray(start)
    for (o, n), m in zip(placed, msgs):
        block[o:o + n] = m
    heap_addr = b.reserve(200)
    block_off = 0
    if root_indirect:
        # the objects sit in the third direct block of the first row
        block_off = 2 * start
        placed = [(o + block_off, n) for o, n in placed]
    dblock = b"FHDB" + bytes([0]) + struct.pack("<Q", heap_addr) + struct.pack("<I", block_off)
    block[:len(dblock)] = dblock
    daddr = b.put(bytes(block))
    if root_indirect:
        children = [U, U, daddr, U]
        iblock = b"FHIB" + bytes([0]) + struct.pack("<Q", heap_addr) + struct.pack("<I", 0)
        iblock += b"".join(struct.pack("<Q", a) for a in children)
        iblock += struct.pack("<I", hdf5.lookup3(iblock))
        root, rows = b.put(iblock), 1
    else:
        root, rows = daddr, 0
    frhp = b"FRHP" + struct.pack("<BHHBI", 0, 7, 0, 0, 4096)
    frhp += struct.pack("<QQQQ", 0, U, 0, U)
    frhp += struct.pack("<QQQQQQ", start, start, 0, len(msgs), 0, 0)
    frhp += struct.pack("<QQ", 0, 0)
    frhp += struct.pack("<HQQHHQH", width, start, max_direct, heap_bits, 1 if root_indirect else 0, root, rows)
    frhp += struct.pack("<I", hdf5.lookup3(frhp))
    b.buf[heap_addr:heap_addr + len(frhp)] = frhp
    recs = b""
    for (n, _), (o, ln) in zip(links, placed):
        heap_id = bytes([0]) + struct.pack("<I", o) + struct.pack("<H", ln)
        recs += struct.pack("<I", hdf5.lookup3(n.encode())) + heap_id
    leaf = b"BTLF" + struct.pack("<BB", 0, 5) + recs
    leaf += struct.pack("<I", hdf5.lookup3(leaf))
    laddr = b.put(leaf)
    bthd = b"BTHD" + struct.pack("<BBIHHBBQHQ", 0, 5, 512, 11, 0, 100, 40, laddr, len(links), len(links))
    bthd += struct.pack("<I", hdf5.lookup3(bthd))
    baddr = b.put(bthd)
    li = struct.pack("<BBQQ", 0, 0, heap_addr, baddr)
    return b.put(ohdr([(hdf5.MSG_LINK_INFO, li, 0), (hdf5.MSG_GROUP_INFO, struct.pack("<BB", 0, 0), 0)]))


@pytest.mark.parametrize("root_indirect", [False, True])
def test_dense_link_storage(tmp_path, root_indirect):
    """More than 8 links in a group written with libver="latest": the link
    messages sit in a fractal heap, found through the name index."""
    b = Builder()
    data = {}
    links = []
    for k in range(12):
        arr = np.full((2, 3), k, dtype=np.int16)
        a = b.put(arr.tobytes())
        links.append((f"frame{k:02d}", dataset(b, arr, struct.pack("<BBQQ", 4, 1, a, arr.nbytes))))
        data[f"frame{k:02d}"] = arr
    g = dense_group(b, links, root_indirect)
    li = struct.pack("<BBQQ", 0, 0, U, U)
    root = b.put(ohdr([(hdf5.MSG_LINK_INFO, li, 0), (hdf5.MSG_LINK, link("frames", g), 0)]))
    path = tmp_path / "dense.h5"
    path.write_bytes(b.finish(root))
    with hdf5.File(path) as f:
        grp = f["frames"]
        assert grp.keys() == sorted(data)
        for k, v in data.items():
            np.testing.assert_array_equal(f[f"frames/{k}"][()], v)
