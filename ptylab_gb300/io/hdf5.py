"""HDF5 reader and writer for PtyLab's measurement and result files.

PtyLab reads its measurement files with PyTables and h5py
(PtyLab/io/readHdf5.py:27-125) and writes its results with h5py
(PtyLab/Reconstruction/Reconstruction.py:510-576); neither library, nor
libhdf5 under them, is part of this package's dependencies.  This module
implements the subset of the published HDF5 file format (format
specification version 3.0) those files use, directly over the bytes:

reading
  * superblock versions 0-3, user blocks of any power-of-two size;
  * object headers version 1 and 2, continuation chunks, committed
    (shared) datatypes;
  * groups stored as symbol tables (version-1 B-tree + local heap; what
    libhdf5 writes by default, MATLAB 7.3 and PyTables included), as compact
    link messages and as dense link storage (a fractal heap with a direct or
    one-level indirect root block, a one-leaf version-2 name index);
  * dataspaces (scalar, simple, null), datatypes: integers, IEEE floats,
    fixed-length strings, bitfields, opaque, compounds (complex numbers
    stored as {r, i} or {real, imag} become numpy complex), enums (h5py's
    booleans become numpy bool), arrays, variable-length strings (str) and
    sequences (numpy arrays) from the global heap;
  * layouts: compact, contiguous, chunked with a version-1 B-tree index or
    (layout version 4) a single chunk, an implicit index or an unpaged fixed
    array; filters deflate, shuffle and fletcher32;
  * attributes (for example MATLAB's ``MATLAB_class``).

writing
  * superblock version 0 with a root symbol-table group, one contiguous
    dataset per name: the classic layout libhdf5 itself writes with its
    default format settings, so h5py, PyTables and MATLAB read it.

Anything outside this subset (larger dense groups, other filters or chunk
indexes) raises ``NotImplementedError`` naming it.
"""

from __future__ import annotations

import os
import struct
import zlib

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF

# message types (format specification section IV.A.2)
MSG_NIL = 0x00
MSG_DATASPACE = 0x01
MSG_LINK_INFO = 0x02
MSG_DATATYPE = 0x03
MSG_FILL_OLD = 0x04
MSG_FILL = 0x05
MSG_LINK = 0x06
MSG_LAYOUT = 0x08
MSG_GROUP_INFO = 0x0A
MSG_PIPELINE = 0x0B
MSG_ATTRIBUTE = 0x0C
MSG_CONTINUATION = 0x10
MSG_SYMBOL_TABLE = 0x11

FILTER_DEFLATE = 1
FILTER_SHUFFLE = 2
FILTER_FLETCHER32 = 3


class HDF5FormatError(ValueError):
    """The file is not HDF5, or its structures are inconsistent."""


# --------------------------------------------------------------------------
# Jenkins lookup3 ("hashlittle"), the checksum of version-2 metadata
# --------------------------------------------------------------------------

def _rot(x, k):
    return ((x << k) | (x >> (32 - k))) & 0xFFFFFFFF


def lookup3(data: bytes, initval: int = 0) -> int:
    """Bob Jenkins' lookup3 ``hashlittle`` (public domain, 2006): the
    checksum HDF5 stores after version-2 superblocks, object headers and
    their continuation chunks."""
    M = 0xFFFFFFFF
    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & M
    i = 0
    while n - i > 12:
        w0, w1, w2 = struct.unpack_from("<3I", data, i)
        a = (a + w0) & M
        b = (b + w1) & M
        c = (c + w2) & M
        a = (a - c) & M; a ^= _rot(c, 4); c = (c + b) & M
        b = (b - a) & M; b ^= _rot(a, 6); a = (a + c) & M
        c = (c - b) & M; c ^= _rot(b, 8); b = (b + a) & M
        a = (a - c) & M; a ^= _rot(c, 16); c = (c + b) & M
        b = (b - a) & M; b ^= _rot(a, 19); a = (a + c) & M
        c = (c - b) & M; c ^= _rot(b, 4); b = (b + a) & M
        i += 12
    if n - i == 0:
        return c
    tail = bytes(data[i:]) + b"\0" * (12 - (n - i))
    w0, w1, w2 = struct.unpack("<3I", tail)
    a = (a + w0) & M
    b = (b + w1) & M
    c = (c + w2) & M
    c ^= b; c = (c - _rot(b, 14)) & M
    a ^= c; a = (a - _rot(c, 11)) & M
    b ^= a; b = (b - _rot(a, 25)) & M
    c ^= b; c = (c - _rot(b, 16)) & M
    a ^= c; a = (a - _rot(c, 4)) & M
    b ^= a; b = (b - _rot(a, 14)) & M
    c ^= b; c = (c - _rot(b, 24)) & M
    return c


# --------------------------------------------------------------------------
# byte cursor
# --------------------------------------------------------------------------

class _Cursor:
    __slots__ = ("buf", "pos")

    def __init__(self, buf, pos=0):
        self.buf = buf
        self.pos = pos

    def u(self, n):
        if self.pos + n > len(self.buf):
            raise HDF5FormatError("structure runs past the end of its block")
        v = int.from_bytes(self.buf[self.pos:self.pos + n], "little")
        self.pos += n
        return v

    def raw(self, n):
        if self.pos + n > len(self.buf):
            raise HDF5FormatError("structure runs past the end of its block")
        v = bytes(self.buf[self.pos:self.pos + n])
        self.pos += n
        return v

    def cstring(self, pad8_from=None):
        end = bytes(self.buf[self.pos:]).find(b"\0")
        if end < 0:
            raise HDF5FormatError("unterminated name")
        s = bytes(self.buf[self.pos:self.pos + end])
        self.pos += end + 1
        if pad8_from is not None:
            used = self.pos - pad8_from
            self.pos += (-used) % 8
        return s

    def skip(self, n):
        self.pos += n


def _parallel(fn, items, threaded):
    """``fn`` over ``items``, on a thread pool when ``threaded`` and there is
    more than a handful of items; the first exception propagates."""
    if not threaded or len(items) < 4:
        for it in items:
            fn(it)
        return
    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=min(len(items), os.cpu_count() or 1, 32)) as ex:
        for _ in ex.map(fn, items):
            pass


def _is_undef(addr, size):
    return addr == (1 << (8 * size)) - 1


# --------------------------------------------------------------------------
# datatypes
# --------------------------------------------------------------------------

_COMPLEX_NAMES = (("r", "i"), ("real", "imag"), ("re", "im"))


def _decode_datatype(cur: _Cursor, reader=None) -> np.dtype:
    """Datatype message (format specification IV.A.2.d) -> numpy dtype."""
    b0 = cur.u(1)
    version, cls = b0 >> 4, b0 & 0x0F
    bits = cur.u(3)
    size = cur.u(4)
    if cls == 0:  # fixed-point
        cur.skip(4)
        order = ">" if bits & 1 else "<"
        return np.dtype(f"{order}{'i' if bits & 0x08 else 'u'}{size}")
    if cls == 1:  # floating point
        off, prec, eloc, esz, mloc, msz, bias = struct.unpack("<HHBBBBI", cur.raw(12))
        if bits & 0x40:
            raise NotImplementedError("VAX floating-point byte order")
        order = ">" if bits & 1 else "<"
        ieee = {2: (10, 5, 10, 15), 4: (23, 8, 23, 127), 8: (52, 11, 52, 1023)}
        if size not in ieee or (eloc, esz, msz, bias) != ieee[size] or off != 0 or mloc != 0:
            raise NotImplementedError(f"non-IEEE floating-point type of {size} bytes")
        return np.dtype(f"{order}f{size}")
    if cls == 3:  # fixed-length string
        return np.dtype(f"S{size}")
    if cls == 4:  # bitfield
        cur.skip(4)
        return np.dtype(f"{'>' if bits & 1 else '<'}u{size}")
    if cls == 5:  # opaque
        taglen = bits & 0xFF
        cur.skip(taglen)
        return np.dtype(f"V{size}")
    if cls == 6:  # compound
        n = bits & 0xFFFF
        names, formats, offsets = [], [], []
        for _ in range(n):
            start = cur.pos
            if version < 3:
                name = cur.cstring(pad8_from=start)
                offset = cur.u(4)
                if version == 1:
                    ndims = cur.u(1)
                    cur.skip(3 + 4 + 4)
                    dims = [cur.u(4) for _ in range(4)]
                    sub = _decode_datatype(cur, reader)
                    if ndims:
                        sub = np.dtype((sub, tuple(dims[:ndims])))
                else:
                    sub = _decode_datatype(cur, reader)
            else:
                name = cur.cstring()
                nb = 1 if size < 1 << 8 else 2 if size < 1 << 16 else 3 if size < 1 << 24 else 4
                offset = cur.u(nb)
                sub = _decode_datatype(cur, reader)
            names.append(name.decode("utf-8"))
            formats.append(sub)
            offsets.append(offset)
        return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": size})
    if cls == 7:  # reference: raw object addresses
        return np.dtype(f"<u{size}")
    if cls == 8:  # enumeration
        n = bits & 0xFFFF
        base = _decode_datatype(cur, reader)
        mnames = []
        for _ in range(n):
            start = cur.pos
            mnames.append(cur.cstring(pad8_from=start if version < 3 else None))
        values = [cur.u(base.itemsize) for _ in range(n)]
        if base.itemsize == 1 and dict(zip(mnames, values)) == {b"FALSE": 0, b"TRUE": 1}:
            return np.dtype(np.bool_)
        return base
    if cls == 9:  # variable length: each element is (length, global heap id)
        kind = bits & 0x0F  # 0 sequence, 1 string
        charset = (bits >> 8) & 0x0F
        base = _decode_datatype(cur, reader)
        so = size - 8
        if so not in (2, 4, 8):
            raise HDF5FormatError(f"variable-length element of {size} bytes")
        return np.dtype([("len", "<u4"), ("addr", f"<u{so}"), ("idx", "<u4")],
                        metadata={"vlen": "str" if kind == 1 else "seq", "base": base, "charset": charset})
    if cls == 10:  # array
        ndims = cur.u(1)
        if version < 3:
            cur.skip(3)
        dims = tuple(cur.u(4) for _ in range(ndims))
        if version < 3:
            cur.skip(4 * ndims)
        base = _decode_datatype(cur, reader)
        return np.dtype((base, dims))
    raise NotImplementedError(f"datatype class {cls}")


def _is_vlen(dt) -> bool:
    return dt.metadata is not None and "vlen" in dt.metadata


def _as_complex(arr: np.ndarray) -> np.ndarray:
    """Compound {r, i} (h5py, PyTables) or {real, imag} (MATLAB) -> complex."""
    dt = arr.dtype
    if dt.names is None or len(dt.names) != 2:
        return arr
    if tuple(dt.names) not in _COMPLEX_NAMES:
        return arr
    f0, f1 = (dt.fields[n] for n in dt.names)
    if f0[0] != f1[0] or f0[0].kind != "f" or f0[1] != 0 or f1[1] != f0[0].itemsize:
        return arr
    ctype = np.dtype(f"{f0[0].byteorder if f0[0].byteorder != '=' else '<'}c{2 * f0[0].itemsize}")
    if dt.itemsize != ctype.itemsize:
        return arr
    return np.ascontiguousarray(arr).view(ctype).astype(ctype.newbyteorder("="), copy=False)


# --------------------------------------------------------------------------
# reader
# --------------------------------------------------------------------------

class _Message:
    __slots__ = ("type", "flags", "data")

    def __init__(self, mtype, flags, data):
        self.type = mtype
        self.flags = flags
        self.data = data


class _Reader:
    def __init__(self, path):
        self.path = str(path)
        self._fh = open(self.path, "rb")
        self.size = os.fstat(self._fh.fileno()).st_size
        try:
            self._read_superblock()
        except Exception:
            self.close()
            raise

    def close(self):
        if self._fh is not None:
            self._fh.close()
            self._fh = None

    # -- primitives --------------------------------------------------------
    def _pread(self, pos, n):
        if pos < 0 or n < 0 or pos + n > self.size:
            raise HDF5FormatError(f"read of {n} bytes at {pos} lies outside the file")
        b = os.pread(self._fh.fileno(), n, pos)
        if len(b) != n:
            raise HDF5FormatError("short read")
        return b

    def at(self, addr, n):
        """``n`` bytes at file address ``addr`` (relative to the base)."""
        return self._pread(self.base + addr, n)

    def cursor(self, addr, n):
        return _Cursor(self.at(addr, n))

    def undef(self, addr):
        return _is_undef(addr, self.so)

    def array_at(self, addr, dtype, count):
        """``count`` elements of ``dtype`` stored contiguously at ``addr``."""
        nbytes = count * dtype.itemsize
        if addr < 0 or self.base + addr + nbytes > self.size:
            raise HDF5FormatError(f"data block at {addr} ({nbytes} bytes) lies outside the file")
        self._fh.seek(self.base + addr)
        arr = np.fromfile(self._fh, dtype=dtype, count=count)
        if arr.size != count:
            raise HDF5FormatError("short read of a data block")
        return arr

    # -- superblock ----------------------------------------------------------
    def _read_superblock(self):
        off = 0
        while off + 8 <= self.size:
            if self._pread(off, 8) == SIGNATURE:
                break
            off = 512 if off == 0 else off * 2
        else:
            raise HDF5FormatError(f"{self.path} is not an HDF5 file (no superblock signature)")
        head = self._pread(off, min(self.size - off, 128))
        c = _Cursor(head, 8)
        version = c.u(1)
        self.superblock_version = version
        if version in (0, 1):
            c.skip(3)  # free-space, root symbol table entry, reserved
            c.skip(1)  # shared header message format
            self.so, self.sl = c.u(1), c.u(1)
            c.skip(1)
            self.leaf_k, self.internal_k = c.u(2), c.u(2)
            c.skip(4)  # consistency flags
            if version == 1:
                c.skip(4)  # indexed storage internal node K, reserved
            base = c.u(self.so)
            c.skip(self.so)  # free-space info
            c.skip(self.so)  # end of file address
            c.skip(self.so)  # driver information block
            c.skip(self.so)  # root: link name offset
            self.root_addr = c.u(self.so)
        elif version in (2, 3):
            self.so, self.sl = c.u(1), c.u(1)
            c.skip(1)
            base = c.u(self.so)
            c.skip(self.so)  # superblock extension
            c.skip(self.so)  # end of file address
            self.root_addr = c.u(self.so)
            end = c.pos
            stored = c.u(4)
            if lookup3(head[:end]) != stored:
                raise HDF5FormatError("superblock checksum mismatch")
        else:
            raise NotImplementedError(f"superblock version {version}")
        if self.so not in (2, 4, 8) or self.sl not in (2, 4, 8):
            raise HDF5FormatError("unsupported sizes of offsets/lengths")
        # addresses are relative to the base address, which is the absolute
        # position of the superblock when the file carries a user block
        self.base = base if base else off

    # -- object headers --------------------------------------------------------
    def messages(self, addr):
        c = self.cursor(addr, min(16, self.size - self.base - addr))
        if c.buf[:4] == b"OHDR":
            return self._messages_v2(addr)
        version = c.u(1)
        if version != 1:
            raise HDF5FormatError(f"object header version {version} at {addr}")
        c.skip(1)
        nmsgs = c.u(2)
        c.skip(4)  # reference count
        hsize = c.u(4)
        chunks = [(addr + 16, hsize)]
        out = []
        seen = 0
        while chunks:
            seen += 1
            if seen > 4096:
                raise HDF5FormatError("object header continuation chain does not end")
            caddr, clen = chunks.pop(0)
            cc = self.cursor(caddr, clen)
            while cc.pos + 8 <= clen:
                mtype, msize, mflags = cc.u(2), cc.u(2), cc.u(1)
                cc.skip(3)
                data = cc.raw(msize)
                if mtype == MSG_CONTINUATION:
                    d = _Cursor(data)
                    chunks.append((d.u(self.so), d.u(self.sl)))
                elif mtype != MSG_NIL:
                    out.append(_Message(mtype, mflags, data))
        del nmsgs
        return out

    def _messages_v2(self, addr):
        c = self.cursor(addr, min(self.size - self.base - addr, 6 + 16 + 4 + 8))
        c.skip(4)
        version = c.u(1)
        if version != 2:
            raise HDF5FormatError(f"object header version {version}")
        flags = c.u(1)
        if flags & 0x20:
            c.skip(16)
        if flags & 0x10:
            c.skip(4)
        chunk0 = c.u(1 << (flags & 3))
        start = c.pos
        body_end = start + chunk0
        c = self.cursor(addr, body_end + 4)
        if lookup3(c.buf[:body_end]) != int.from_bytes(c.buf[body_end:body_end + 4], "little"):
            raise HDF5FormatError(f"object header checksum mismatch at {addr}")
        chunks = [(c.buf, start, body_end)]
        out = []
        hdr = 4 + (2 if flags & 0x04 else 0)
        while chunks:
            buf, pos, end = chunks.pop(0)
            cc = _Cursor(buf, pos)
            while cc.pos + hdr <= end:
                mtype, msize, mflags = cc.u(1), cc.u(2), cc.u(1)
                if flags & 0x04:
                    cc.skip(2)
                data = cc.raw(msize)
                if mtype == MSG_CONTINUATION:
                    d = _Cursor(data)
                    caddr, clen = d.u(self.so), d.u(self.sl)
                    blk = self.at(caddr, clen)
                    if blk[:4] != b"OCHK":
                        raise HDF5FormatError("bad object header continuation signature")
                    if lookup3(blk[:clen - 4]) != int.from_bytes(blk[clen - 4:clen], "little"):
                        raise HDF5FormatError("object header continuation checksum mismatch")
                    chunks.append((blk, 4, clen - 4))
                elif mtype != MSG_NIL:
                    out.append(_Message(mtype, mflags, data))
        return out

    def shared_datatype(self, data):
        """A shared datatype message: the datatype of the committed object
        the message points to."""
        c = _Cursor(data)
        version = c.u(1)
        kind = c.u(1)
        if version == 1:
            c.skip(6)
        elif version == 3 and kind != 2:
            raise NotImplementedError("datatypes in the shared object header message heap")
        addr = c.u(self.so)
        for m in self.messages(addr):
            if m.type == MSG_DATATYPE:
                return _decode_datatype(_Cursor(m.data), self)
        raise HDF5FormatError("committed datatype without a datatype message")

    def datatype(self, msg):
        if msg.flags & 0x02:
            return self.shared_datatype(msg.data)
        return _decode_datatype(_Cursor(msg.data), self)

    # -- groups ------------------------------------------------------------------
    def local_heap(self, addr):
        c = self.cursor(addr, 8 + 2 * self.sl + self.so)
        if c.raw(4) != b"HEAP":
            raise HDF5FormatError("bad local heap signature")
        c.skip(4)
        dsize = c.u(self.sl)
        c.skip(self.sl)
        daddr = c.u(self.so)
        return self.at(daddr, dsize)

    def group_links(self, msgs):
        """Name -> object header address for a group's members."""
        links = {}
        for m in msgs:
            if m.type == MSG_SYMBOL_TABLE:
                c = _Cursor(m.data)
                btree, heap = c.u(self.so), c.u(self.so)
                names = self.local_heap(heap)
                self._walk_group_btree(btree, names, links, depth=0)
            elif m.type == MSG_LINK_INFO:
                c = _Cursor(m.data)
                c.skip(1)
                flags = c.u(1)
                if flags & 1:
                    c.skip(8)
                fheap = c.u(self.so)
                names_bt = c.u(self.so)
                if not self.undef(fheap):
                    for data in self._dense_link_messages(fheap, names_bt):
                        name, addr = self._decode_link(data)
                        if addr is not None:
                            links[name] = addr
            elif m.type == MSG_LINK:
                name, addr = self._decode_link(m.data)
                if addr is not None:
                    links[name] = addr
        return links

    # -- dense link storage: a fractal heap of link messages, indexed by a
    # version-2 B-tree of name hashes (format specification III.G, III.A.2)
    def _dense_link_messages(self, heap_addr, btree_addr):
        heap = self._fractal_heap(heap_addr)
        for heap_id in self._btree2_records(btree_addr, id_len=heap["id_len"]):
            yield self._heap_object(heap, heap_id)

    def _fractal_heap(self, addr):
        c = self.cursor(addr, 4 + 1 + 2 + 2 + 1 + 4 + 12 * max(self.so, self.sl) + 2 + 2 * self.sl + 2 + 2 + self.so + 2)
        if c.raw(4) != b"FRHP":
            raise HDF5FormatError("bad fractal heap signature")
        c.skip(1)
        h = {"id_len": c.u(2)}
        filters_len = c.u(2)
        c.skip(1)  # flags
        h["max_obj"] = c.u(4)
        c.skip(self.sl)  # next huge object id
        c.skip(self.so)  # huge object B-tree
        c.skip(self.sl)  # free space in managed blocks
        c.skip(self.so)  # free space manager
        c.skip(6 * self.sl)  # managed space, allocated, iterator, managed/huge/tiny counts and sizes (first six)
        c.skip(2 * self.sl)  # tiny objects: size and count
        h["width"] = c.u(2)
        h["start"] = c.u(self.sl)
        h["max_direct"] = c.u(self.sl)
        h["max_heap_bits"] = c.u(2)
        c.skip(2)  # starting rows in the root indirect block
        h["root"] = c.u(self.so)
        h["root_rows"] = c.u(2)
        if filters_len:
            raise NotImplementedError("filtered fractal heaps")
        # heap id fields: the offset in bytes for max_heap_bits; the length
        # in the smaller of the bytes for an offset inside the largest direct
        # block and the bytes that encode the largest managed object
        h["off_bytes"] = (h["max_heap_bits"] + 7) // 8
        dir_bytes = ((h["max_direct"].bit_length() - 1) + 7) // 8
        obj_bytes = (h["max_obj"].bit_length() - 1) // 8 + 1
        h["len_bytes"] = max(1, min(dir_bytes, obj_bytes))
        return h

    def _btree2_records(self, addr, id_len):
        c = self.cursor(addr, 4 + 1 + 1 + 4 + 2 + 2 + 1 + 1 + self.so + 2 + self.sl)
        if c.raw(4) != b"BTHD":
            raise HDF5FormatError("bad version-2 B-tree signature")
        c.skip(1)
        btype = c.u(1)
        c.skip(4)  # node size
        rec_size = c.u(2)
        depth = c.u(2)
        c.skip(2)
        root = c.u(self.so)
        nrec = c.u(2)
        if btype != 5:
            raise NotImplementedError(f"version-2 B-tree of type {btype} for links")
        if depth != 0:
            raise NotImplementedError("link name index deeper than one leaf")
        if self.undef(root) or nrec == 0:
            return []
        leaf = self.cursor(root, 6 + nrec * rec_size)
        if leaf.raw(4) != b"BTLF":
            raise HDF5FormatError("bad version-2 B-tree leaf signature")
        leaf.skip(2)
        out = []
        for _ in range(nrec):
            leaf.skip(4)  # name hash
            out.append(leaf.raw(id_len))
            leaf.skip(rec_size - 4 - id_len)
        return out

    def _heap_object(self, h, heap_id):
        kind = (heap_id[0] >> 4) & 3
        if kind == 2:  # tiny: the object is in the id
            n = (heap_id[0] & 0x0F) + 1
            return bytes(heap_id[1:1 + n])
        if kind != 0:
            raise NotImplementedError("huge objects in a fractal heap")
        cur = _Cursor(heap_id, 1)
        off = cur.u(h["off_bytes"])
        n = cur.u(h["len_bytes"])
        if h["root_rows"] == 0:  # the root is one direct block holding offsets from 0
            return self.at(h["root"] + off, n)
        # root indirect block: rows of `width` direct blocks (start, start,
        # 2 start, 4 start, ...); children listed row by row
        width, start = h["width"], h["start"]
        c = self.cursor(h["root"], 5 + self.so + h["off_bytes"] + h["root_rows"] * width * self.so)
        if c.raw(4) != b"FHIB":
            raise HDF5FormatError("bad fractal heap indirect block signature")
        c.skip(1 + self.so + h["off_bytes"])
        block_off = 0
        for row in range(h["root_rows"]):
            size = start if row < 2 else start << (row - 1)
            if size > h["max_direct"]:
                raise NotImplementedError("fractal heap with nested indirect blocks")
            for _ in range(width):
                child = c.u(self.so)
                if block_off <= off < block_off + size:
                    if self.undef(child):
                        raise HDF5FormatError("heap object in an unallocated block")
                    return self.at(child + off - block_off, n)
                block_off += size
        raise HDF5FormatError("heap offset beyond the root indirect block")

    def _walk_group_btree(self, addr, names, links, depth):
        if depth > 32:
            raise HDF5FormatError("group B-tree deeper than 32 levels")
        c = self.cursor(addr, 8 + 2 * self.so)
        if c.raw(4) != b"TREE":
            raise HDF5FormatError("bad B-tree signature")
        ntype, level, entries = c.u(1), c.u(1), c.u(2)
        if ntype != 0:
            raise HDF5FormatError("group B-tree of the wrong node type")
        c = self.cursor(addr + 8 + 2 * self.so, (2 * entries + 1) * max(self.sl, self.so))
        children = []
        for _ in range(entries):
            c.skip(self.sl)  # key: heap offset
            children.append(c.u(self.so))
        for child in children:
            if level > 0:
                self._walk_group_btree(child, names, links, depth + 1)
            else:
                self._read_snod(child, names, links)

    def _read_snod(self, addr, names, links):
        c = self.cursor(addr, 8)
        if c.raw(4) != b"SNOD":
            raise HDF5FormatError("bad symbol table node signature")
        c.skip(2)
        nsyms = c.u(2)
        esize = 2 * self.so + 24
        c = self.cursor(addr + 8, nsyms * esize)
        for _ in range(nsyms):
            noff = c.u(self.so)
            oaddr = c.u(self.so)
            c.skip(24)
            nc = _Cursor(names, noff)
            links[nc.cstring().decode("utf-8")] = oaddr

    def _decode_link(self, data):
        c = _Cursor(data)
        c.skip(1)
        flags = c.u(1)
        ltype = c.u(1) if flags & 0x08 else 0
        if flags & 0x04:
            c.skip(8)
        if flags & 0x10:
            c.skip(1)
        nlen = c.u(1 << (flags & 3))
        name = c.raw(nlen).decode("utf-8")
        if ltype != 0:  # soft or external link: not followed
            return name, None
        return name, c.u(self.so)

    # -- datasets ----------------------------------------------------------------
    def dataspace(self, data):
        c = _Cursor(data)
        version = c.u(1)
        rank = c.u(1)
        flags = c.u(1)
        if version == 1:
            c.skip(5)
            kind = 1 if rank else 0
        elif version == 2:
            kind = c.u(1)
        else:
            raise NotImplementedError(f"dataspace version {version}")
        if kind == 2:
            return None
        return tuple(c.u(self.sl) for _ in range(rank))

    def global_heap_object(self, addr, index):
        """Object ``index`` of the global heap collection at ``addr``."""
        cache = self.__dict__.setdefault("_gcol", {})
        if addr not in cache:
            head = self.cursor(addr, 8 + self.sl)
            if head.raw(4) != b"GCOL":
                raise HDF5FormatError("bad global heap signature")
            head.skip(4)
            size = head.u(self.sl)
            c = self.cursor(addr, size)
            c.skip(8 + self.sl)
            objs = {}
            while c.pos + 8 + self.sl <= size:
                idx = c.u(2)
                c.skip(6)
                n = c.u(self.sl)
                if idx == 0:
                    break
                objs[idx] = c.raw(n)
                c.skip((-n) % 8)
            cache[addr] = objs
        try:
            return cache[addr][index]
        except KeyError:
            raise HDF5FormatError(f"global heap object {index} missing") from None

    def resolve_vlen(self, arr):
        """(length, heap id) records -> an object array of str (strings) or
        numpy arrays of the base type (sequences)."""
        meta = arr.dtype.metadata
        base = meta["base"]
        out = np.empty(arr.shape, dtype=object)
        flat = arr.reshape(-1)
        res = out.reshape(-1)
        for k in range(flat.size):
            n, addr, idx = int(flat[k]["len"]), int(flat[k]["addr"]), int(flat[k]["idx"])
            if meta["vlen"] == "str":
                raw = self.global_heap_object(addr, idx)[:n] if n else b""
                res[k] = raw.rstrip(b"\0").decode("utf-8" if meta["charset"] == 1 else "ascii", errors="replace")
            else:
                raw = self.global_heap_object(addr, idx) if n else b""
                res[k] = np.frombuffer(raw, dtype=base, count=n).copy()
        return out

    def read_fill(self, msgs, dtype):
        for m in msgs:
            if m.type == MSG_FILL:
                c = _Cursor(m.data)
                version = c.u(1)
                value = None
                if version in (1, 2):
                    c.skip(2)
                    defined = c.u(1)
                    if version == 1 or defined:
                        n = c.u(4) if c.pos + 4 <= len(c.buf) else 0
                        if n:
                            value = c.raw(n)
                elif version == 3:
                    flags = c.u(1)
                    if flags & 0x20:
                        n = c.u(4)
                        value = c.raw(n)
                if value is not None and len(value) == dtype.itemsize:
                    return np.frombuffer(value, dtype=dtype)[0]
        return None

    def read_dataset(self, msgs):
        shape = dtype = layout = None
        filters = []
        for m in msgs:
            if m.type == MSG_DATASPACE:
                shape = self.dataspace(m.data)
            elif m.type == MSG_DATATYPE:
                dtype = self.datatype(m)
            elif m.type == MSG_LAYOUT:
                layout = m.data
            elif m.type == MSG_PIPELINE:
                filters = self._pipeline(m.data)
        if dtype is None or layout is None:
            raise HDF5FormatError("dataset without a datatype or layout message")
        if shape is None:
            return np.empty((0,), dtype=dtype)
        nelem = int(np.prod(shape, dtype=np.int64)) if shape else 1
        nbytes = nelem * dtype.itemsize
        c = _Cursor(layout)
        version = c.u(1)
        if version in (1, 2):
            ndims = c.u(1)
            cls = c.u(1)
            c.skip(5)
            addr = c.u(self.so) if cls != 0 else None
            dims = [c.u(4) for _ in range(ndims)]
            if cls == 0:
                n = c.u(4)
                arr = np.frombuffer(c.raw(n), dtype=dtype, count=nelem)
            elif cls == 1:
                arr = self._contiguous(addr, nbytes, dtype, nelem)
            else:
                esize = c.u(4)
                arr = self._chunked_btree(addr, shape, dtype, dims[:-1] if len(dims) > len(shape) else dims,
                                          filters, msgs, esize)
        elif version in (3, 4):
            cls = c.u(1)
            if cls == 0:
                n = c.u(2)
                arr = np.frombuffer(c.raw(n), dtype=dtype, count=nelem)
            elif cls == 1:
                addr = c.u(self.so)
                c.skip(self.sl)
                arr = self._contiguous(addr, nbytes, dtype, nelem)
            elif cls == 2 and version == 3:
                ndims = c.u(1)
                addr = c.u(self.so)
                dims = [c.u(4) for _ in range(ndims)]
                arr = self._chunked_btree(addr, shape, dtype, dims[:-1], filters, msgs, dims[-1])
            elif cls == 2:
                arr = self._chunked_v4(c, shape, dtype, filters, msgs)
            elif cls == 3:
                raise NotImplementedError("virtual datasets")
            else:
                raise HDF5FormatError(f"layout class {cls}")
        else:
            raise NotImplementedError(f"layout message version {version}")
        arr = np.asarray(arr).reshape(shape)
        if _is_vlen(dtype):
            return self.resolve_vlen(arr)
        return _as_complex(arr)

    def _contiguous(self, addr, nbytes, dtype, nelem):
        if self.undef(addr):  # storage never allocated: all fill value
            return np.zeros(nelem, dtype=dtype)
        return self.array_at(addr, dtype, nelem)

    def _pipeline(self, data):
        c = _Cursor(data)
        version = c.u(1)
        n = c.u(1)
        if version == 1:
            c.skip(6)
        out = []
        for _ in range(n):
            fid = c.u(2)
            nlen = c.u(2) if (version == 1 or fid >= 256) else 0
            flags = c.u(2)
            nvals = c.u(2)
            name = c.raw(nlen) if nlen else b""
            vals = [c.u(4) for _ in range(nvals)]
            if version == 1 and nvals % 2:
                c.skip(4)
            out.append((fid, flags, name.rstrip(b"\0").decode("latin-1"), vals))
        return out

    def _unfilter(self, raw, filters, mask):
        for i in range(len(filters) - 1, -1, -1):
            if mask & (1 << i):
                continue
            fid, _, name, vals = filters[i]
            if fid == FILTER_DEFLATE:
                raw = zlib.decompress(raw)
            elif fid == FILTER_SHUFFLE:
                es = vals[0] if vals else 1
                n = len(raw) // es
                if es > 1 and n > 1:
                    body = np.frombuffer(raw, np.uint8, count=n * es).reshape(es, n).T.tobytes()
                    raw = body + raw[n * es:]
            elif fid == FILTER_FLETCHER32:
                raw = raw[:-4]
            else:
                raise NotImplementedError(f"HDF5 filter {fid} ({name or 'unnamed'})")
        return raw

    def _place_chunk(self, out, raw, offsets, chunk, dtype):
        block = np.frombuffer(raw, dtype=dtype, count=int(np.prod(chunk))).reshape(chunk)
        dst, src = [], []
        for o, cdim, sdim in zip(offsets, chunk, out.shape):
            n = min(cdim, sdim - o)
            if n <= 0:
                return
            dst.append(slice(o, o + n))
            src.append(slice(0, n))
        out[tuple(dst)] = block[tuple(src)]

    def _new_output(self, shape, dtype, msgs):
        out = np.zeros(shape, dtype=dtype)
        fill = self.read_fill(msgs, dtype)
        if fill is not None:
            out[...] = fill
        return out

    def _chunked_btree(self, addr, shape, dtype, chunk, filters, msgs, esize):
        out = self._new_output(shape, dtype, msgs)
        if self.undef(addr):
            return out
        rank = len(shape)
        chunk = tuple(chunk[:rank])
        nbytes = int(np.prod(chunk)) * dtype.itemsize
        stack = [(addr, 0)]
        pending = []
        while stack:
            node, depth = stack.pop()
            if depth > 64:
                raise HDF5FormatError("chunk B-tree deeper than 64 levels")
            c = self.cursor(node, 8 + 2 * self.so)
            if c.raw(4) != b"TREE":
                raise HDF5FormatError("bad chunk B-tree signature")
            ntype, level, entries = c.u(1), c.u(1), c.u(2)
            if ntype != 1:
                raise HDF5FormatError("chunk B-tree of the wrong node type")
            ksize = 8 + 8 * (rank + 1)
            c = self.cursor(node + 8 + 2 * self.so, entries * (ksize + self.so) + ksize)
            for _ in range(entries):
                csize = c.u(4)
                mask = c.u(4)
                offs = [c.u(8) for _ in range(rank + 1)][:rank]
                child = c.u(self.so)
                if level > 0:
                    stack.append((child, depth + 1))
                    continue
                pending.append((child, csize, mask, offs))
        self._decode_chunks(out, pending, filters, chunk, dtype, nbytes)
        return out

    def _decode_chunks(self, out, pending, filters, chunk, dtype, nbytes):
        """Read, unfilter and place chunks; filtered chunks are decoded on a
        thread pool (zlib and the byte shuffles release the GIL)."""

        # shuffle applied first on writing is undone last on reading: when the
        # chunk lies wholly inside the output and its destination is
        # contiguous, undo it straight into the destination (one strided copy)
        last_shuffle = bool(filters) and filters[0][0] == FILTER_SHUFFLE and dtype.itemsize > 1

        def one(item):
            child, csize, mask, offs = item
            raw = self.at(child, csize)
            if last_shuffle and not mask & 1:
                raw = self._unfilter(raw, filters[1:], mask >> 1)
                if len(raw) < nbytes:
                    raise HDF5FormatError("chunk shorter than its shape")
                dst = tuple(slice(o, o + c) for o, c in zip(offs, chunk))
                dest = out[dst] if all(o + c <= s for o, c, s in zip(offs, chunk, out.shape)) else None
                if dest is not None and dest.flags.c_contiguous:
                    es = filters[0][3][0] if filters[0][3] else dtype.itemsize
                    n = nbytes // es
                    if es == dtype.itemsize and n * es == nbytes:
                        planes = np.frombuffer(raw, np.uint8, count=nbytes).reshape(es, n)
                        dest.view(np.uint8).reshape(n, es)[...] = planes.T
                        return
                raw = self._unfilter(raw, filters[:1], 0)
            elif filters:
                raw = self._unfilter(raw, filters, mask)
            if len(raw) < nbytes:
                raise HDF5FormatError("chunk shorter than its shape")
            self._place_chunk(out, raw, offs, chunk, dtype)

        _parallel(one, pending, bool(filters))

    def _chunked_v4(self, c, shape, dtype, filters, msgs):
        flags = c.u(1)
        ndims = c.u(1)
        enc = c.u(1)
        dims = [c.u(enc) for _ in range(ndims)]
        chunk = tuple(dims[:len(shape)])
        itype = c.u(1)
        out = self._new_output(shape, dtype, msgs)
        rank = len(shape)
        grid = [-(-s // k) for s, k in zip(shape, chunk)]
        nbytes = int(np.prod(chunk)) * dtype.itemsize
        if itype == 1:  # single chunk
            fsize = mask = None
            if flags & 0x02:
                fsize = c.u(self.sl)
                mask = c.u(4)
            addr = c.u(self.so)
            if self.undef(addr):
                return out
            raw = bytes(self.at(addr, fsize if fsize is not None else nbytes))
            if filters:
                raw = self._unfilter(raw, filters, mask or 0)
            self._place_chunk(out, raw, [0] * rank, chunk, dtype)
            return out
        if itype == 2:  # implicit: unfiltered chunks in row-major order
            addr = c.u(self.so)
            if self.undef(addr):
                return out
            for k, idx in enumerate(np.ndindex(*grid)):
                raw = bytes(self.at(addr + k * nbytes, nbytes))
                self._place_chunk(out, raw, [i * ck for i, ck in zip(idx, chunk)], chunk, dtype)
            return out
        if itype == 3:  # fixed array
            c.skip(1)  # page bits
            addr = c.u(self.so)
            if self.undef(addr):
                return out
            entries = self._fixed_array(addr, filtered=bool(filters))
            pending = [(caddr, csize if csize is not None else nbytes, mask, [i * ck for i, ck in zip(idx, chunk)])
                       for idx, (caddr, csize, mask) in zip(np.ndindex(*grid), entries) if not self.undef(caddr)]
            self._decode_chunks(out, pending, filters, chunk, dtype, nbytes)
            return out
        raise NotImplementedError({4: "extensible-array chunk index",
                                   5: "version-2 B-tree chunk index"}.get(itype, f"chunk index {itype}"))

    def _fixed_array(self, addr, filtered):
        c = self.cursor(addr, 8 + self.sl + self.so + 4)
        if c.raw(4) != b"FAHD":
            raise HDF5FormatError("bad fixed array header signature")
        c.skip(1)
        client = c.u(1)
        esize = c.u(1)
        page_bits = c.u(1)
        n = c.u(self.sl)
        daddr = c.u(self.so)
        if n > (1 << page_bits):
            raise NotImplementedError("paged fixed-array chunk index")
        d = self.cursor(daddr, 6 + self.so + n * esize + 4)
        if d.raw(4) != b"FADB":
            raise HDF5FormatError("bad fixed array data block signature")
        d.skip(2)
        d.skip(self.so)
        out = []
        for _ in range(n):
            if client == 0:
                out.append((d.u(self.so), None, 0))
            else:
                caddr = d.u(self.so)
                csize = d.u(esize - self.so - 4)
                out.append((caddr, csize, d.u(4)))
        return out

    def attributes(self, msgs):
        attrs = {}
        for m in msgs:
            if m.type != MSG_ATTRIBUTE:
                continue
            c = _Cursor(m.data)
            version = c.u(1)
            c.skip(1)
            nsz, tsz, ssz = c.u(2), c.u(2), c.u(2)
            if version == 3:
                c.skip(1)
            pad = (lambda n: n + (-n) % 8) if version == 1 else (lambda n: n)
            name = c.raw(pad(nsz))[:nsz].rstrip(b"\0").decode("utf-8")
            tbytes = c.raw(pad(tsz))
            sbytes = c.raw(pad(ssz))
            try:
                dt = _decode_datatype(_Cursor(tbytes), self)
                shape = self.dataspace(sbytes)
            except NotImplementedError:
                continue
            if shape is None:
                attrs[name] = None
                continue
            n = int(np.prod(shape, dtype=np.int64)) if shape else 1
            val = np.frombuffer(c.raw(n * dt.itemsize), dtype=dt, count=n).reshape(shape)
            if _is_vlen(dt):
                v = self.resolve_vlen(val)
                attrs[name] = v[()] if shape == () else v
                continue
            val = _as_complex(val)
            attrs[name] = val[()] if shape == () else val.copy()
        return attrs


class Dataset:
    """A dataset of an open file.  ``ds[()]`` / ``np.array(ds)`` / ``read()``
    return the whole array (complex compounds as numpy complex)."""

    def __init__(self, reader, addr, name, msgs):
        self._reader = reader
        self._addr = addr
        self._msgs = msgs
        self.name = name
        self.shape = None
        for m in msgs:
            if m.type == MSG_DATASPACE:
                self.shape = reader.dataspace(m.data)
        self.attrs = reader.attributes(msgs)

    @property
    def dtype(self):
        for m in self._msgs:
            if m.type == MSG_DATATYPE:
                dt = self._reader.datatype(m)
                return np.dtype(object) if _is_vlen(dt) else _as_complex(np.empty(0, dt)).dtype
        raise HDF5FormatError("dataset without a datatype")

    def read(self):
        return self._reader.read_dataset(self._msgs)

    def __getitem__(self, key):
        arr = self.read()
        return arr if key is Ellipsis else arr[key]

    def __array__(self, dtype=None, copy=None):
        arr = self.read()
        return arr if dtype is None else arr.astype(dtype)

    def __len__(self):
        if not self.shape:
            raise TypeError("scalar dataset has no length")
        return self.shape[0]


class Group:
    """A group of an open file: a read-only mapping of names to groups and
    datasets, in name order."""

    def __init__(self, reader, addr, name="/", msgs=None):
        self._reader = reader
        self.name = name
        msgs = reader.messages(addr) if msgs is None else msgs
        self._links = dict(sorted(reader.group_links(msgs).items()))
        self.attrs = reader.attributes(msgs)

    def keys(self):
        return list(self._links)

    def __iter__(self):
        return iter(self._links)

    def __len__(self):
        return len(self._links)

    def __contains__(self, path):
        try:
            self[path]
        except KeyError:
            return False
        return True

    def __getitem__(self, path):
        node = self
        parts = [p for p in str(path).split("/") if p]
        if not parts:
            return self
        for i, part in enumerate(parts):
            if not isinstance(node, Group) or part not in node._links:
                raise KeyError(f"{path!r} not found in {self._reader.path}")
            addr = node._links[part]
            msgs = self._reader.messages(addr)
            full = "/" + "/".join(parts[:i + 1])
            if any(m.type == MSG_LAYOUT for m in msgs):
                node = Dataset(self._reader, addr, full, msgs)
            else:
                node = Group(self._reader, addr, full, msgs)
        return node

    def items(self):
        return [(k, self[k]) for k in self._links]

    def values(self):
        return [self[k] for k in self._links]


# --------------------------------------------------------------------------
# writer
# --------------------------------------------------------------------------

_LEAF_K = 4        # symbols per symbol-table node: 2 * leaf K
_INTERNAL_K = 16   # children per group B-tree node: 2 * internal K
_SNOD_SIZE = 8 + 2 * _LEAF_K * 40
_BTREE_SIZE = 24 + (2 * _INTERNAL_K + 1) * 8 + 2 * _INTERNAL_K * 8
_MAX_NAMES = 2 * _INTERNAL_K * 2 * _LEAF_K


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * ((-len(b)) % 8)


def _encode_datatype(dt: np.dtype) -> bytes:
    """numpy dtype -> datatype message (class/version byte, 3 bit-field
    bytes, size, properties), in the versions libhdf5 writes by default."""
    dt = np.dtype(dt)
    if dt.kind == "b":
        base = _encode_datatype(np.dtype("i1"))
        names = _pad8(b"FALSE\0") + _pad8(b"TRUE\0")
        return struct.pack("<B3sI", 0x18, (2).to_bytes(3, "little"), 1) + base + names + b"\x00\x01"
    if dt.kind in "iu":
        bits = (0x08 if dt.kind == "i" else 0) | (1 if dt.byteorder == ">" else 0)
        return struct.pack("<B3sIHH", 0x10, bits.to_bytes(3, "little"), dt.itemsize, 0, 8 * dt.itemsize)
    if dt.kind == "f":
        layout = {2: (15, 10, 5, 10, 15), 4: (31, 23, 8, 23, 127), 8: (63, 52, 11, 52, 1023)}
        if dt.itemsize not in layout:
            raise NotImplementedError(f"floating-point type {dt}")
        sign, eloc, esz, msz, bias = layout[dt.itemsize]
        bits = 0x20 | (sign << 8) | (1 if dt.byteorder == ">" else 0)
        return struct.pack("<B3sIHHBBBBI", 0x11, bits.to_bytes(3, "little"), dt.itemsize,
                           0, 8 * dt.itemsize, eloc, esz, 0, msz, bias)
    if dt.kind == "c":
        half = np.dtype(f"{dt.byteorder if dt.byteorder in '<>' else '<'}f{dt.itemsize // 2}")
        member = _encode_datatype(half)
        body = b""
        for name, off in ((b"r", 0), (b"i", half.itemsize)):
            body += _pad8(name + b"\0") + struct.pack("<IB3xI4x4I", off, 0, 0, 0, 0, 0, 0) + member
        return struct.pack("<B3sI", 0x16, (2).to_bytes(3, "little"), dt.itemsize) + body
    if dt.kind == "S":
        return struct.pack("<B3sI", 0x13, (1).to_bytes(3, "little"), dt.itemsize)
    raise NotImplementedError(f"writing datatype {dt}")


def _message_v1(mtype, data, flags=0):
    data = _pad8(data)
    return struct.pack("<HHB3x", mtype, len(data), flags) + data


def _object_header_v1(messages):
    body = b"".join(messages)
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body


_CHUNK_K = 32  # indexed-storage B-tree K of a version-0 superblock: 2K chunks per node


class _Storage:
    """Where one dataset's elements go: a contiguous block, or encoded
    chunks indexed by a version-1 B-tree (type 1)."""

    def __init__(self, arr, chunks=None, filters=()):
        self.arr = arr
        self.chunks = chunks
        self.filters = list(filters)
        self.blocks = []     # (offset, bytes), offsets relative to the storage start
        self.nodes = []
        self.size = 0
        self.root = None     # relative offset of the B-tree root
        if chunks is None:
            self.size = arr.nbytes
            return
        rank = arr.ndim
        grid = [-(-s // c) for s, c in zip(arr.shape, chunks)]
        origins = [[i * c for i, c in zip(idx, chunks)] for idx in np.ndindex(*grid)]
        encoded = [None] * len(origins)

        def encode(k):
            origin = origins[k]
            block = np.zeros(chunks, dtype=arr.dtype)
            src = tuple(slice(o, min(o + c, s)) for o, c, s in zip(origin, chunks, arr.shape))
            block[tuple(slice(0, x.stop - x.start) for x in src)] = arr[src]
            raw = block.tobytes()
            for fid, vals in self.filters:
                if fid == FILTER_SHUFFLE and vals[0] > 1:
                    raw = np.frombuffer(raw, np.uint8).reshape(-1, vals[0]).T.tobytes()
                elif fid == FILTER_DEFLATE:
                    raw = zlib.compress(raw, vals[0])
            encoded[k] = raw

        _parallel(encode, list(range(len(origins))), bool(self.filters))
        entries = [(o, self._put(raw), len(raw)) for o, raw in zip(origins, encoded)]
        if not entries:
            return
        keysize = 8 + 8 * (rank + 1)
        nodesize = 24 + 2 * _CHUNK_K * 8 + (2 * _CHUNK_K + 1) * keysize

        def key(origin, nbytes):
            return struct.pack("<II", nbytes, 0) + b"".join(struct.pack("<Q", o) for o in origin) + bytes(8)

        right = key([o + c for o, c in zip(entries[-1][0], chunks)], 0)
        self.nodesize = nodesize
        self.nodes = []      # (offset, level, [(key, child offset)], left, right, last key)
        level, children = 0, [(key(o, n), a) for o, a, n in entries]
        while True:
            groups = [children[i:i + 2 * _CHUNK_K] for i in range(0, len(children), 2 * _CHUNK_K)]
            addrs = [self._reserve(nodesize) for _ in groups]
            parents = []
            for g, (grp, a) in enumerate(zip(groups, addrs)):
                left = addrs[g - 1] if g else None
                nxt = addrs[g + 1] if g + 1 < len(addrs) else None
                last = groups[g + 1][0][0] if g + 1 < len(groups) else right
                self.nodes.append((a, level, grp, left, nxt, last))
                parents.append((grp[0][0], a))
            if len(parents) == 1:
                self.root = parents[0][1]
                break
            level += 1
            if level > 8:
                raise NotImplementedError("chunk index deeper than 8 levels")
            children = parents

    def _put(self, raw):
        a = self._reserve(len(raw))
        self.blocks.append((a, raw))
        return a

    def _reserve(self, n):
        self.size += (-self.size) % 8
        a = self.size
        self.size += n
        return a

    def layout(self, base):
        if self.chunks is None:
            return struct.pack("<BBQQ", 3, 1, base if self.size else UNDEF, self.arr.nbytes)
        root = UNDEF if self.root is None else base + self.root
        return (struct.pack("<BBBQ", 3, 2, self.arr.ndim + 1, root)
                + b"".join(struct.pack("<I", c) for c in self.chunks)
                + struct.pack("<I", self.arr.dtype.itemsize))

    def pipeline(self):
        if not self.filters:
            return None
        body = struct.pack("<BB6x", 1, len(self.filters))
        for fid, vals in self.filters:
            body += struct.pack("<HHHH", fid, 0, 1, len(vals)) + b"".join(struct.pack("<I", v) for v in vals)
            if len(vals) % 2:
                body += bytes(4)
        return body

    def write(self, fh, base):
        if self.chunks is None:
            if self.size:
                fh.seek(base)
                fh.write(memoryview(self.arr).cast("B"))
            return
        for off, raw in self.blocks:
            fh.seek(base + off)
            fh.write(raw)
        rel = lambda a: UNDEF if a is None else base + a
        for off, level, grp, left, nxt, last in self.nodes:
            node = bytearray(b"TREE" + struct.pack("<BBHQQ", 1, level, len(grp), rel(left), rel(nxt)))
            for k, child in grp:
                node += k + struct.pack("<Q", base + child)
            node += last
            node += bytes(self.nodesize - len(node))
            fh.seek(base + off)
            fh.write(node)


class _Writer:
    def __init__(self, path):
        self.path = str(path)
        self.items = {}

    def add(self, name, data, dtype=None, chunks=None, compression=None, compression_opts=None,
            shuffle=False):
        if not isinstance(name, str) or not name or "/" in name.strip("/"):
            raise ValueError(f"dataset name {name!r}: only datasets in the root group are written")
        name = name.strip("/")
        if name in self.items:
            raise ValueError(f"dataset {name!r} already exists")
        arr = np.asarray(data)
        if dtype is not None:
            arr = arr.astype(np.dtype(dtype))
        if arr.dtype.kind == "U":
            arr = np.char.encode(arr, "utf-8")
        if arr.dtype.kind == "O":
            raise NotImplementedError("writing object (variable-length) arrays")
        arr = np.asarray(arr, order="C")  # keeps 0-d arrays 0-d
        if arr.dtype.byteorder == ">" or (arr.dtype.byteorder == "=" and np.little_endian is False):
            arr = arr.astype(arr.dtype.newbyteorder("<"))
        _encode_datatype(arr.dtype)  # fail before the file is touched
        filters = []
        if shuffle:
            filters.append((FILTER_SHUFFLE, [arr.dtype.itemsize]))
        if compression is not None:
            if compression not in ("gzip", FILTER_DEFLATE):
                raise NotImplementedError(f"compression {compression!r}: only gzip is written")
            level = 4 if compression_opts is None else int(compression_opts)
            if not 0 <= level <= 9:
                raise ValueError("gzip level must lie in 0..9")
            filters.append((FILTER_DEFLATE, [level]))
        if filters and chunks is None:
            chunks = True
        if chunks is True:
            chunks = _auto_chunks(arr.shape, arr.dtype.itemsize)
        if chunks is not None:
            chunks = tuple(int(c) for c in chunks)
            if arr.ndim == 0 or len(chunks) != arr.ndim or any(c < 1 for c in chunks):
                raise ValueError(f"chunk shape {chunks} does not fit data of shape {arr.shape}")
            if arr.dtype.itemsize * int(np.prod(chunks)) >= 1 << 32:
                raise ValueError("chunks must hold less than 4 GiB")
        self.items[name] = _Storage(arr, chunks, filters)

    def write(self):
        names = sorted(self.items, key=lambda s: s.encode("utf-8"))
        if len(names) > _MAX_NAMES:
            raise NotImplementedError(f"more than {_MAX_NAMES} datasets in one file")
        # local heap: "" at offset 0, then the names, then one free block
        heap = bytearray(8)
        name_off = {}
        for n in names:
            name_off[n] = len(heap)
            heap += _pad8(n.encode("utf-8") + b"\0")
        free_off = len(heap)
        free_size = 16 + 8 * max(0, 8 - len(names))
        heap += struct.pack("<QQ", 1, free_size) + b"\0" * (free_size - 16)
        snods = [names[i:i + 2 * _LEAF_K] for i in range(0, len(names), 2 * _LEAF_K)]

        addr = 96
        heap_hdr = addr
        heap_data = heap_hdr + 32
        addr = heap_data + len(heap)
        btree = addr
        addr += _BTREE_SIZE
        snod_addr = []
        for _ in snods:
            snod_addr.append(addr)
            addr += _SNOD_SIZE
        root_hdr = addr
        root_msgs = [_message_v1(MSG_SYMBOL_TABLE, struct.pack("<QQ", btree, heap_hdr), flags=1)]
        root_blob = _object_header_v1(root_msgs)
        addr += len(root_blob)

        # dataset object headers, then each dataset's storage (16-byte aligned)
        hdr_addr, blobs, data_addr = {}, {}, {}
        for n in names:
            hdr_addr[n] = addr
            addr += len(self._dataset_header(self.items[n], 0))
        for n in names:
            addr += (-addr) % 16
            data_addr[n] = addr
            addr += self.items[n].size
        eof = addr
        for n in names:
            blobs[n] = self._dataset_header(self.items[n], data_addr[n])

        out = bytearray()
        out += SIGNATURE
        out += struct.pack("<BBBBBBBB", 0, 0, 0, 0, 0, 8, 8, 0)
        out += struct.pack("<HHI", _LEAF_K, _INTERNAL_K, 0)
        out += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
        out += struct.pack("<QQII", 0, root_hdr, 1, 0) + struct.pack("<QQ", btree, heap_hdr)
        out += b"HEAP" + bytes(4) + struct.pack("<QQQ", len(heap), free_off, heap_data)
        out += heap
        node = bytearray(b"TREE" + struct.pack("<BBH", 0, 0, len(snods)) + struct.pack("<QQ", UNDEF, UNDEF))
        node += struct.pack("<Q", 0)
        for group, a in zip(snods, snod_addr):
            node += struct.pack("<QQ", a, name_off[group[-1]])
        node += bytes(_BTREE_SIZE - len(node))
        out += node
        for group in snods:
            s = bytearray(b"SNOD" + struct.pack("<BBH", 1, 0, len(group)))
            for n in group:
                s += struct.pack("<QQII", name_off[n], hdr_addr[n], 0, 0) + bytes(16)
            s += bytes(_SNOD_SIZE - len(s))
            out += s
        out += root_blob
        for n in names:
            out += blobs[n]
        if len(out) != (hdr_addr[names[-1]] + len(blobs[names[-1]]) if names else root_hdr + len(root_blob)):
            raise AssertionError("metadata layout mismatch")
        with open(self.path, "wb") as fh:
            fh.write(out)
            for n in names:
                self.items[n].write(fh, data_addr[n])
            fh.truncate(eof)

    def _dataset_header(self, st, data_addr):
        arr = st.arr
        space = struct.pack("<BBB5x", 1, arr.ndim, 0) + b"".join(struct.pack("<Q", d) for d in arr.shape)
        msgs = [_message_v1(MSG_DATASPACE, space), _message_v1(MSG_DATATYPE, _encode_datatype(arr.dtype), flags=1)]
        pipe = st.pipeline()
        if pipe is not None:
            msgs.append(_message_v1(MSG_PIPELINE, pipe))
        msgs.append(_message_v1(MSG_LAYOUT, st.layout(data_addr)))
        return _object_header_v1(msgs)


def _auto_chunks(shape, itemsize, target=1 << 20):
    """A chunk shape of about ``target`` bytes: whole trailing dimensions
    (one detector frame per chunk for a ptychogram), halved from the front
    while larger."""
    chunks = [max(1, int(s)) for s in shape]
    i = 0
    while int(np.prod(chunks)) * itemsize > target and i < len(chunks):
        if chunks[i] > 1:
            chunks[i] = -(-chunks[i] // 2)
        else:
            i += 1
    return tuple(chunks)


# --------------------------------------------------------------------------
# public entry point
# --------------------------------------------------------------------------

class File(Group):
    """``File(path)`` / ``File(path, "r")`` opens an HDF5 file for reading;
    ``File(path, "w")`` collects ``create_dataset`` calls and writes the file
    when closed (or at the end of a ``with`` block).  The read side is a
    :class:`Group` for the root group."""

    def __init__(self, path, mode="r"):
        self.mode = mode
        self.filename = str(path)
        if mode == "r":
            self._writer = None
            reader = _Reader(path)
            try:
                super().__init__(reader, reader.root_addr, "/")
            except Exception:
                reader.close()
                raise
        elif mode == "w":
            self._writer = _Writer(path)
            self._reader = None
            self._links = {}
            self.attrs = {}
            self.name = "/"
        else:
            raise ValueError(f"mode {mode!r}: only 'r' and 'w' are supported")

    def create_dataset(self, name, data=None, dtype=None, chunks=None, compression=None,
                       compression_opts=None, shuffle=False):
        """h5py's ``create_dataset`` for data given in full: contiguous by
        default; ``chunks`` (a shape or True), ``compression="gzip"`` with
        ``compression_opts`` (level, default 4) and ``shuffle`` store it in
        chunks."""
        if self._writer is None:
            raise ValueError("file is open for reading")
        self._writer.add(name, data, dtype, chunks, compression, compression_opts, shuffle)

    def __setitem__(self, name, data):
        self.create_dataset(name, data=data)

    def keys(self):
        if self._writer is not None:
            return sorted(self._writer.items)
        return super().keys()

    def close(self):
        if self._writer is not None:
            w, self._writer = self._writer, None
            w.write()
        elif self._reader is not None:
            self._reader.close()

    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc, tb):
        if exc_type is not None and self._writer is not None:
            self._writer = None  # leave no half-described file behind
            return False
        self.close()
        return False


def is_hdf5(path) -> bool:
    """True when ``path`` carries the HDF5 signature at 0, 512, 1024, ..."""
    try:
        size = os.path.getsize(path)
        with open(path, "rb") as fh:
            off = 0
            while off + 8 <= size:
                fh.seek(off)
                if fh.read(8) == SIGNATURE:
                    return True
                off = 512 if off == 0 else off * 2
    except OSError:
        return False
    return False
