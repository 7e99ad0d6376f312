"""A small writer of MATLAB -v7.3 MAT-files (HDF5 behind MATLAB's 512-byte user
block), for testing the library's reader without h5py or MATLAB.

Written from the HDF5 file format specification (version 3.0), with the
structures MATLAB's save -v7.3 produces: a version 0 superblock, version 1
object headers and a root group held in a symbol table (version 1 B-tree,
symbol table nodes, local heap); numeric arrays as datasets with the MATLAB
dimensions reversed and a MATLAB_class attribute, complex arrays as compounds
{real, imag}, structs as groups.  `new_style=True` writes the newer forms
instead: a version 2 superblock, version 2 object headers ("OHDR"), link
messages, version 2 dataspaces and version 3 attributes.  Checksums of the
version 2 structures are written as zeros (the reader does not verify them).

Datasets can be contiguous, compact or chunked (version 1 B-tree of chunks, one
or two levels; or a version 4 layout with a single chunk), with the deflate
(1), shuffle (2) and Fletcher-32 (3) filters applied in the order given.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIG = b"\x89HDF\r\n\x1a\n"
DEFLATE, SHUFFLE, FLETCHER32 = 1, 2, 3


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * (-len(b) % 8)


def _q(*v) -> bytes:
    return struct.pack("<%dQ" % len(v), *v)


# ---- datatypes ----------------------------------------------------------------

def dt_float(size: int, be: bool = False) -> bytes:
    bits0 = (1 if be else 0) | 0x20  # byte order, mantissa normalisation "implied msb"
    if size == 4:
        props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
    else:
        props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
    return struct.pack("<BBBBI", 0x11, bits0, 8 * size - 1, 0, size) + props


def dt_int(size: int, signed: bool, be: bool = False) -> bytes:
    bits0 = (1 if be else 0) | (0x08 if signed else 0)
    return struct.pack("<BBBBI", 0x10, bits0, 0, 0, size) + struct.pack("<HH", 0, 8 * size)


def dt_string(n: int) -> bytes:
    return struct.pack("<BBBBI", 0x13, 0, 0, 0, n)


def dt_complex(size: int, be: bool = False, version: int = 1) -> bytes:
    """Compound {real, imag} of two IEEE floats of `size` bytes each."""
    m = dt_float(size, be)
    out = struct.pack("<BHBI", (version << 4) | 6, 2, 0, 2 * size)
    for name, off in ((b"real", 0), (b"imag", size)):
        if version == 1:
            out += _pad8(name + b"\0") + struct.pack("<IB3xI4x", off, 0, 0) + b"\0" * 16 + m
        elif version == 2:
            out += _pad8(name + b"\0") + struct.pack("<I", off) + m
        else:
            out += name + b"\0" + bytes([off]) + m
    return out


def numpy_type(arr: np.ndarray, be: bool) -> tuple[bytes, np.dtype, int]:
    """(HDF5 datatype message, numpy element type in the file's byte order, bytes)."""
    k, s = arr.dtype.kind, arr.dtype.itemsize
    o = ">" if be else "<"
    if k == "f":
        return dt_float(s, be), np.dtype(o + "f%d" % s), s
    if k == "c":
        h = s // 2
        return (dt_complex(h, be), np.dtype([("real", o + "f%d" % h), ("imag", o + "f%d" % h)]),
                s)
    if k in "iu":
        return dt_int(s, k == "i", be), np.dtype(o + k + str(s)), s
    if k == "b":
        return dt_int(1, False, be), np.dtype("u1"), 1
    raise TypeError(arr.dtype)


# ---- messages --------------------------------------------------------------------

def dataspace(dims, version: int = 1, maxdims: bool = True) -> bytes:
    dims = list(dims)
    body = b"".join(_q(d) for d in dims)
    if maxdims:
        body += b"".join(_q(d) for d in dims)
    if version == 1:
        return struct.pack("<BBB5x", 1, len(dims), 1 if maxdims else 0) + body
    return struct.pack("<BBBB", 2, len(dims), 1 if maxdims else 0, 1 if dims else 0) + body


def attribute(name: str, dt: bytes, ds: bytes, data: bytes, version: int = 1) -> bytes:
    nm = name.encode() + b"\0"
    if version == 1:
        return (struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(ds)) + _pad8(nm) + _pad8(dt)
                + _pad8(ds) + data)
    return struct.pack("<BBHHHB", 3, 0, len(nm), len(dt), len(ds), 0) + nm + dt + ds + data


def class_attr(mclass: str, version: int = 1) -> bytes:
    scalar = dataspace([], version=1 if version == 1 else 2, maxdims=False)
    return attribute("MATLAB_class", dt_string(len(mclass)), scalar, mclass.encode(), version)


def filters_msg(fs, version: int = 1) -> bytes:
    if version == 1:
        out = struct.pack("<BB6x", 1, len(fs))
        for fid in fs:
            vals = [4] if fid == SHUFFLE else ([6] if fid == DEFLATE else [])
            out += struct.pack("<HHHH", fid, 0, 0, len(vals)) + b"".join(
                struct.pack("<I", v) for v in vals)
            if len(vals) % 2:
                out += b"\0" * 4
        return out
    out = struct.pack("<BB", 2, len(fs))
    for fid in fs:
        vals = [4] if fid == SHUFFLE else ([6] if fid == DEFLATE else [])
        out += struct.pack("<HHH", fid, 0, len(vals)) + b"".join(struct.pack("<I", v) for v in vals)
    return out


def shuffle(b: bytes, es: int) -> bytes:
    n = len(b) // es
    a = np.frombuffer(b[: n * es], np.uint8).reshape(n, es)
    return a.T.tobytes() + b[n * es:]


def apply_filters(b: bytes, fs, es: int) -> bytes:
    for fid in fs:
        if fid == SHUFFLE:
            b = shuffle(b, es)
        elif fid == DEFLATE:
            b = zlib.compress(b, 6)
        elif fid == FLETCHER32:
            b = b + b"\x01\x02\x03\x04"  # the reader drops the checksum unverified
    return b


# ---- the file --------------------------------------------------------------------

class Mat73Writer:
    def __init__(self, new_style: bool = False, userblock: int = 512):
        self.new = new_style
        self.b = bytearray()
        if userblock:
            txt = (b"MATLAB 7.3 MAT-file, Platform: GLNXA64, Created on: Fri Dec  4 12:00:00 2026 "
                   b"HDF5 schema 1.00 .")
            hdr = txt.ljust(116, b" ") + b"\0" * 8 + struct.pack("<H", 0x0200) + b"IM"
            self.b += hdr.ljust(userblock, b"\0")
        self.sb = len(self.b)
        self.b += b"\0" * (48 if new_style else 96)
        self.links: list[tuple[str, int]] = []

    # addresses are relative to the superblock
    def _put(self, data: bytes) -> int:
        while len(self.b) % 8:
            self.b.append(0)
        off = len(self.b)
        self.b += data
        return off - self.sb

    def _header(self, msgs, cont_split: int | None = None) -> int:
        """Object header of (type, data) messages; messages from cont_split on go
        to a continuation block."""
        if cont_split is not None:
            first, rest = msgs[:cont_split], msgs[cont_split:]
            blk = self._block(rest)
            first = first + [(0x10, _q(blk[0], blk[1]))]
            msgs = first
        if self.new:
            body = b"".join(struct.pack("<BHB", t, len(d), 0) + d for t, d in msgs)
            return self._put(b"OHDR" + bytes([2, 2]) + struct.pack("<I", len(body)) + body +
                             b"\0" * 4)
        body = b"".join(struct.pack("<HHB3x", t, len(_pad8(d)), 0) + _pad8(d) for t, d in msgs)
        return self._put(struct.pack("<BBHII4x", 1, 0, len(msgs), 1, len(body)) + body)

    def _block(self, msgs):
        """A continuation block of messages: (address, length)."""
        if self.new:
            body = b"".join(struct.pack("<BHB", t, len(d), 0) + d for t, d in msgs)
            data = b"OCHK" + body + b"\0" * 4
        else:
            data = b"".join(struct.pack("<HHB3x", t, len(_pad8(d)), 0) + _pad8(d) for t, d in msgs)
        return self._put(data), len(data)

    def _attrs(self, mclass, extra=()):
        v = 3 if self.new else 1
        out = []
        if mclass:
            out.append((0x0C, class_attr(mclass, v)))
        for name, dt, data in extra:
            scalar = dataspace([], version=1 if v == 1 else 2, maxdims=False)
            out.append((0x0C, attribute(name, dt, scalar, data, v)))
        return out

    def add(self, name: str, arr, mclass: str | None = None, layout: str = "contiguous",
            chunks=None, filters=(), be: bool = False, levels: int = 1, skip_mask_chunk=None,
            continuation: bool = False, empty_dims=None):
        """A variable: arr in MATLAB order (column-major dims), stored with its
        dimensions reversed.  layout: contiguous, compact, chunked (version 1
        B-tree of `levels` levels) or single (version 4 layout, one chunk).
        chunks: chunk dimensions in the file's (reversed) order.  empty_dims: an
        empty MATLAB array of these dimensions (MATLAB_empty: the data are the
        dimensions)."""
        extra = []
        if empty_dims is not None:
            arr = np.asarray(empty_dims, dtype=np.uint64)
            extra.append(("MATLAB_empty", dt_int(1, False), b"\x01"))
        arr = np.asarray(arr)
        if mclass is None:
            mclass = {"f8": "double", "f4": "single", "c16": "double", "c8": "single",
                      "b1": "logical"}.get(arr.dtype.kind + str(arr.dtype.itemsize),
                                           arr.dtype.name)
        dt, npt, es = numpy_type(arr, be)
        hdims = list(arr.shape[::-1])
        h = np.ascontiguousarray(arr.T)  # the file's row-major view
        if arr.dtype.kind == "c":
            rec = np.empty(h.shape, npt)
            rec["real"], rec["imag"] = h.real, h.imag
            raw_arr = rec
        else:
            raw_arr = h.astype(npt)
        ds = dataspace(hdims, version=2 if self.new else 1)
        msgs = [(0x01, ds), (0x03, dt)]
        if layout == "contiguous":
            raw = raw_arr.tobytes()
            msgs.append((0x08, struct.pack("<BB", 3, 1) + _q(self._put(raw), len(raw))))
        elif layout == "compact":
            raw = raw_arr.tobytes()
            msgs.append((0x08, struct.pack("<BBH", 3, 0, len(raw)) + raw))
        elif layout in ("chunked", "single"):
            chunks = list(chunks if chunks is not None else hdims)
            if filters:
                msgs.append((0x0B, filters_msg(filters, 2 if self.new else 1)))
            grid = [range(0, d, c) for d, c in zip(hdims, chunks)]
            entries = []
            for idx in np.ndindex(*[len(g) for g in grid]):
                o = [g[i] for g, i in zip(grid, idx)]
                block = np.zeros(chunks, npt)
                sl = tuple(slice(a, min(a + c, d)) for a, c, d in zip(o, chunks, hdims))
                part = raw_arr[sl]
                block[tuple(slice(0, s) for s in part.shape)] = part
                mask = 0
                fs = list(filters)
                if skip_mask_chunk is not None and tuple(o) == tuple(skip_mask_chunk):
                    mask = 1 << fs.index(DEFLATE)  # this chunk stored without deflate
                    fs = [f for f in fs if f != DEFLATE]
                data = apply_filters(block.tobytes(), fs, es)
                entries.append((o, len(data), mask, self._put(data)))
            if layout == "single":
                assert len(entries) == 1
                o, size, mask, addr = entries[0]
                flags = 0x02 if filters else 0
                body = struct.pack("<BBBBB", 4, 2, flags, len(chunks) + 1, 4) + b"".join(
                    struct.pack("<I", c) for c in chunks + [es]) + bytes([1])
                if filters:
                    body += struct.pack("<QI", size, mask)
                msgs.append((0x08, body + _q(addr)))
            else:
                bt = self._chunk_tree(entries, len(hdims), levels)
                msgs.append((0x08, struct.pack("<BBB", 3, 2, len(chunks) + 1) + _q(bt) + b"".join(
                    struct.pack("<I", c) for c in chunks + [es])))
        else:
            raise ValueError(layout)
        msgs += self._attrs(mclass, extra)
        hdr = self._header(msgs, cont_split=len(msgs) - 1 if continuation else None)
        self.links.append((name, hdr))

    def _chunk_tree(self, entries, rank, levels):
        def key(o, size=0, mask=0):
            return struct.pack("<II", size, mask) + b"".join(_q(x) for x in list(o) + [0])

        def node(level, items, end_key):
            out = b"TREE" + struct.pack("<BBH", 1, level, len(items)) + _q(UNDEF, UNDEF)
            for k, child in items:
                out += k + _q(child)
            return self._put(out + end_key)

        end = key([UNDEF & 0xFFFFFFFF] * rank)
        leaves = [(key(o, s, m), a) for o, s, m, a in entries]
        if levels == 1:
            return node(0, leaves, end)
        half = max(1, len(leaves) // 2)
        parts = [leaves[:half], leaves[half:]] if len(leaves) > 1 else [leaves]
        kids = [(p[0][0], node(0, p, end)) for p in parts if p]
        return node(1, kids, end)

    def add_group(self, name: str, mclass: str | None = "struct"):
        """An (empty) group, as MATLAB stores structs and cells."""
        if self.new:
            msgs = [(0x02, struct.pack("<BB", 0, 0) + _q(UNDEF, UNDEF))]
        else:
            heap, _ = self._heap([])
            bt = self._put(b"TREE" + struct.pack("<BBH", 0, 0, 0) + _q(UNDEF, UNDEF) + _q(0))
            msgs = [(0x11, _q(bt, heap))]
        msgs += self._attrs(mclass)
        self.links.append((name, self._header(msgs)))

    def _heap(self, names):
        data = bytearray(b"\0" * 8)
        offs = []
        for n in names:
            offs.append(len(data))
            data += _pad8(n.encode() + b"\0")
        dseg = self._put(bytes(data))
        return self._put(b"HEAP" + struct.pack("<B3x", 0) + _q(len(data), 1, dseg)), offs

    def save(self, path, dense: bool = False, per_node: int | None = None):
        """per_node (old style): symbol table nodes of at most this many entries,
        under a two-level group B-tree (a level-1 root over two level-0 nodes)."""
        links = sorted(self.links)
        if self.new:
            msgs = [(0x02, struct.pack("<BB", 0, 0) + _q(self._put(b"FRHP") if dense else UNDEF,
                                                           UNDEF))]
            for name, hdr in links:
                nm = name.encode()
                msgs.append((0x06, struct.pack("<BBB", 1, 0, len(nm)) + nm + _q(hdr)))
            root = self._header(msgs)
            eof = len(self.b) - self.sb
            sb = SIG + struct.pack("<BBBB", 2, 8, 8, 0) + _q(0, UNDEF, eof, root) + b"\0" * 4
        else:
            heap, offs = self._heap([n for n, _ in links])
            ent = [struct.pack("<QQII", off, hdr, 0, 0) + b"\0" * 16
                   for off, (_, hdr) in zip(offs, links)]
            # symbol table nodes (keys: heap offsets of each node's last name)
            if per_node is None:
                half = max(1, len(ent) // 2)
                groups = [ent[:half], ent[half:]] if len(ent) > 1 else [ent]
            else:
                groups = [ent[i:i + per_node] for i in range(0, len(ent), per_node)]
            snods, keys = [], [0]
            start = 0
            for g in groups:
                snods.append(self._put(b"SNOD" + struct.pack("<BBH", 1, 0, len(g)) + b"".join(g)))
                start += len(g)
                keys.append(offs[start - 1] if offs else 0)

            def tree(level, children, ks):
                body = b"TREE" + struct.pack("<BBH", 0, level, len(children)) + _q(UNDEF, UNDEF)
                for k, c in zip(ks, children):
                    body += _q(k, c)
                return self._put(body + _q(ks[len(children)]))

            if per_node is None or len(snods) < 2:
                bt = tree(0, snods, keys)
            else:  # two level-0 nodes under a level-1 root
                h = len(snods) // 2
                left = tree(0, snods[:h], keys[:h + 1])
                right = tree(0, snods[h:], keys[h:])
                bt = tree(1, [left, right], [keys[0], keys[h], keys[-1]])
            root = self._header([(0x11, _q(bt, heap))])
            eof = len(self.b) - self.sb
            sb = (SIG + struct.pack("<BBBBBBBB", 0, 0, 0, 0, 0, 8, 8, 0) +
                  struct.pack("<HHI", 4, 16, 0) + _q(0, UNDEF, eof, UNDEF) +
                  struct.pack("<QQII", 0, root, 1, 0) + _q(bt, heap))
        self.b[self.sb:self.sb + len(sb)] = sb
        with open(path, "wb") as f:
            f.write(bytes(self.b))
