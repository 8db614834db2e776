"""A minimal writer of HDF5 files in the format's earliest layout (test helper).

The reference's SOFA fixtures use version-2 object headers and dense
groups.  Files written by older HDF5 releases (the layout of many SOFA
files from the Matlab API) use a version-0 superblock, version-1 object
headers, a symbol-table group (version-1 B-tree, local heap), and
attribute and dataspace messages of version 1.  This writer produces that
layout, following the published file format specification, so that
tests/test_hdf5_layouts.py can read it back with sparrowpy_gb300.hdf5:

* datasets: contiguous, compact, or chunked (version-1 B-tree of chunks,
  optional shuffle + deflate, edge chunks padded as HDF5 stores them), and
  chunked with a version-4 layout message (single-chunk, implicit or
  fixed-array index);
* types: little-endian float64, int32, fixed-length strings and
  variable-length strings (global heap);
* attributes on the root group and on datasets.
"""
import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


def _pad8(b):
    return b + b"\x00" * ((-len(b)) % 8)


def _dtype_msg(kind, size=0):
    if kind == "f8":
        return bytes([0x11, 0x20, 63, 0]) + struct.pack("<I", 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
    if kind == "i4":
        return bytes([0x10, 0x08, 0, 0]) + struct.pack("<I", 4) + struct.pack("<HH", 0, 32)
    if kind == "str":
        return bytes([0x13, 0x00, 0, 0]) + struct.pack("<I", size)
    if kind == "vlstr":
        base = bytes([0x10, 0x00, 0, 0]) + struct.pack("<I", 1) + struct.pack("<HH", 0, 8)
        return bytes([0x19, 0x01, 0, 0]) + struct.pack("<I", 16) + base
    raise ValueError(kind)


def _space_msg(shape):
    return bytes([1, len(shape), 0, 0]) + b"\x00" * 4 + b"".join(struct.pack("<Q", d) for d in shape)


class Writer:
    """Collects objects, then lays the file out in one pass (addresses are known when writing)."""

    def __init__(self):
        self.buf = bytearray(96)  # the superblock, written last
        self.gheap = []           # variable-length strings: (index, bytes)

    def _alloc(self, data):
        addr = len(self.buf)
        self.buf += _pad8(bytes(data))
        return addr

    def _header(self, messages):
        """A version-1 object header holding (type, data) messages."""
        body = b""
        for mtype, data in messages:
            data = _pad8(data)
            body += struct.pack("<HHB3x", mtype, len(data), 0) + data
        return self._alloc(struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body)

    def _vl_ref(self, text):
        self.gheap.append(text.encode())
        return len(self.gheap)  # index within the collection (1-based); the address is patched later

    def _attr_msg(self, name, value):
        nm = name.encode() + b"\x00"
        if isinstance(value, str) and value.startswith("vl:"):
            text = value[3:]
            dt, sp = _dtype_msg("vlstr"), _space_msg(())
            data = struct.pack("<I", len(text.encode())) + b"GHEAPADR" + struct.pack("<I", self._vl_ref(text))
        elif isinstance(value, str):
            raw = value.encode()
            dt, sp, data = _dtype_msg("str", len(raw)), _space_msg(()), raw
        else:
            arr = np.asarray(value, dtype="<f8")
            dt, sp, data = _dtype_msg("f8"), _space_msg(arr.shape), arr.tobytes()
        head = struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(sp))
        return 0x0C, head + _pad8(nm) + _pad8(dt) + _pad8(sp) + data

    def dataset(self, array, layout="contiguous", chunks=None, filters=False, attrs=None):
        """Write a dataset; returns its object header address."""
        a = np.ascontiguousarray(array)
        kind = {"f": "f8", "i": "i4"}[a.dtype.kind]
        a = a.astype("<f8" if kind == "f8" else "<i4")
        msgs = [(0x01, _space_msg(a.shape)), (0x03, _dtype_msg(kind))]
        esz = a.dtype.itemsize
        if layout.startswith("v4-"):
            return self._header(msgs + self._v4_layout(a, layout[3:], chunks, filters, esz) +
                                [self._attr_msg(k, v) for k, v in (attrs or {}).items()])
        if layout == "compact":
            raw = a.tobytes()
            msgs.append((0x08, struct.pack("<BBH", 3, 0, len(raw)) + raw))
        elif layout == "contiguous":
            addr = self._alloc(a.tobytes())
            msgs.append((0x08, struct.pack("<BBQQ", 3, 1, addr, a.nbytes)))
        else:
            rank = a.ndim
            chunk_list = []
            grid = [-(-a.shape[i] // chunks[i]) for i in range(rank)]
            for idx in np.ndindex(*grid):
                block = np.zeros(chunks, dtype=a.dtype)  # edge chunks are stored whole, padded
                src = tuple(slice(i * c, min((i + 1) * c, s)) for i, c, s in zip(idx, chunks, a.shape))
                block[tuple(slice(0, sl.stop - sl.start) for sl in src)] = a[src]
                raw = block.tobytes()
                if filters:
                    raw = np.frombuffer(raw, np.uint8).reshape(-1, esz).T.tobytes()  # shuffle
                    raw = zlib.compress(raw)
                chunk_list.append((tuple(i * c for i, c in zip(idx, chunks)), self._alloc(raw), len(raw)))
            nd = rank + 1
            node = b"TREE" + struct.pack("<BBHQQ", 1, 0, len(chunk_list), UNDEF, UNDEF)
            for offs, addr, size in chunk_list:
                node += struct.pack("<II", size, 0) + b"".join(struct.pack("<Q", o) for o in offs + (0,))
                node += struct.pack("<Q", addr)
            node += struct.pack("<II", 0, 0) + b"".join(struct.pack("<Q", s) for s in a.shape + (0,))
            btree = self._alloc(node)
            msgs.append((0x08, struct.pack("<BBBQ", 3, 2, nd, btree) +
                         b"".join(struct.pack("<I", c) for c in tuple(chunks) + (esz,))))
            if filters:
                shuffle = struct.pack("<HHHH", 2, 0, 0, 1) + struct.pack("<I", esz) + b"\x00" * 4
                deflate = struct.pack("<HHHH", 1, 0, 0, 1) + struct.pack("<I", 6) + b"\x00" * 4
                msgs.append((0x0B, struct.pack("<BB6x", 1, 2) + shuffle + deflate))
        for name, value in (attrs or {}).items():
            msgs.append(self._attr_msg(name, value))
        return self._header(msgs)

    def _v4_layout(self, a, index, chunks, filters, esz):
        """Layout message version 4 with a single-chunk, implicit or fixed-array chunk index (checksums are
        written as zeros: the reader does not check them)."""
        chunks = tuple(a.shape) if index == "single" else tuple(chunks)
        grid = [-(-a.shape[i] // chunks[i]) for i in range(a.ndim)]
        stored = []
        for idx in np.ndindex(*grid):
            block = np.zeros(chunks, dtype=a.dtype)
            src = tuple(slice(i * c, min((i + 1) * c, s)) for i, c, s in zip(idx, chunks, a.shape))
            block[tuple(slice(0, sl.stop - sl.start) for sl in src)] = a[src]
            raw = block.tobytes()
            if filters:
                raw = zlib.compress(np.frombuffer(raw, np.uint8).reshape(-1, esz).T.tobytes())
            stored.append(raw)
        dims = b"".join(struct.pack("<I", c) for c in chunks + (esz,))
        flags = 0x02 if (filters and index == "single") else 0
        head = struct.pack("<BBBBB", 4, 2, flags, a.ndim + 1, 4) + dims
        msgs = []
        if index == "single":
            addr = self._alloc(stored[0])
            info = (struct.pack("<QI", len(stored[0]), 0) if filters else b"") + struct.pack("<Q", addr)
            msgs.append((0x08, head + bytes([1]) + info))
        elif index == "implicit":
            assert not filters
            addr = self._alloc(b"".join(stored))
            msgs.append((0x08, head + bytes([2]) + struct.pack("<Q", addr)))
        else:  # fixed array: client 1 (filtered) holds address, 4-byte size and mask; client 0 the address
            addrs = [self._alloc(raw) for raw in stored]
            client, esize = (1, 16) if filters else (0, 8)
            hdr_addr = len(self.buf)
            dblock_addr = hdr_addr + 32
            hdr = b"FAHD" + struct.pack("<BBBBQQ", 0, client, esize, 10, len(stored), dblock_addr) + b"\x00" * 4
            self._alloc(hdr)
            assert len(self.buf) == dblock_addr
            elems = b"".join(struct.pack("<QII", ad, len(raw), 0) if filters else struct.pack("<Q", ad)
                             for ad, raw in zip(addrs, stored))
            self._alloc(b"FADB" + struct.pack("<BBQ", 0, client, hdr_addr) + elems + b"\x00" * 4)
            msgs.append((0x08, head + bytes([3, 10]) + struct.pack("<Q", hdr_addr)))
        if filters:
            shuffle = struct.pack("<HHHH", 2, 0, 0, 1) + struct.pack("<I", esz) + b"\x00" * 4
            deflate = struct.pack("<HHHH", 1, 0, 0, 1) + struct.pack("<I", 6) + b"\x00" * 4
            msgs.append((0x0B, struct.pack("<BB6x", 1, 2) + shuffle + deflate))
        return msgs

    def finish(self, path, links, root_attrs=None):
        """Write the root group (symbol table of `links`: name -> header address) and the file."""
        names = b"\x00" * 8
        offsets = {}
        for name in links:
            offsets[name] = len(names)
            names += _pad8(name.encode() + b"\x00")
        heap_data = self._alloc(names)
        heap = self._alloc(b"HEAP" + struct.pack("<B3xQQQ", 0, len(names), UNDEF, heap_data))
        entries = b"".join(struct.pack("<QQII16x", offsets[n], addr, 0, 0) for n, addr in sorted(links.items()))
        snod = self._alloc(b"SNOD" + struct.pack("<BBH", 1, 0, len(links)) + entries)
        last = max(offsets.values()) if offsets else 0
        tree = self._alloc(b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, UNDEF, UNDEF) + struct.pack("<QQQ", 0, snod, last))
        msgs = [(0x11, struct.pack("<QQ", tree, heap))]
        for name, value in (root_attrs or {}).items():
            msgs.append(self._attr_msg(name, value))
        root = self._header(msgs)
        if self.gheap:  # the global heap collection, then the variable-length references point at it
            objs = b""
            for k, data in enumerate(self.gheap, start=1):
                objs += struct.pack("<HH4xQ", k, 1, len(data)) + _pad8(data)
            size = max(4096, 16 + len(objs) + 16)
            col = b"GCOL" + struct.pack("<B3xQ", 1, size) + objs
            col += struct.pack("<HH4xQ", 0, 0, size - len(col) - 16)
            col += b"\x00" * (size - len(col))
            gaddr = self._alloc(col)
            self.buf = self.buf.replace(b"GHEAPADR", struct.pack("<Q", gaddr))
        eof = len(self.buf)
        sb = b"\x89HDF\r\n\x1a\n" + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
        sb += struct.pack("<QQII", 0, root, 1, 0) + struct.pack("<QQ", tree, heap)
        assert len(sb) == 96
        self.buf[:96] = sb
        with open(path, "wb") as fh:
            fh.write(bytes(self.buf))
