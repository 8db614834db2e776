"""A reader for the subset of HDF5 that SOFA files use (netCDF-4 files).

sparrowpy reads SOFA files through sofar, which reads them through netCDF4
and the HDF5 library (sound_object.py:26, classes/RadiosityKang.py:574).
None of those is installed here, so this module reads the HDF5 container
itself, following the published HDF5 file format specification (version 3
of the format document): superblocks of versions 0 to 3; object headers of
versions 1 and 2 with continuation blocks; groups held in symbol tables
(version-1 B-trees, local heaps), in link messages, or densely (fractal
heap plus version-2 B-tree name index); attributes in object headers or
dense storage; dataspaces; fixed-point, floating-point, fixed-length
string and variable-length string types (global heap); contiguous, compact
and chunked layouts (version-1 B-tree, single-chunk, implicit and
fixed-array chunk indexes) with the deflate, shuffle and Fletcher-32
filters.  Anything else raises ``NotImplementedError`` naming the
feature, so an unsupported file fails loudly instead of decoding wrongly.

Checked against real files (sparrowpy's SOFA test data): superblocks of
versions 0 and 2, version-2 object headers, dense link and attribute
storage, chunked data under version-1 B-trees with shuffle and deflate,
fixed-length string attributes.  Version-1 object headers, symbol-table
groups, variable-length strings, compact layouts and multi-chunk data with
padded edge chunks are checked against files that a small writer of the
same specification produces (the test suite's hdf5_earliest.py), not
against files of the HDF5 library; so are the version-4 chunk indexes
(single chunk, implicit, fixed array).

Only what the radiosity path needs is exposed: ``File(path)`` with
``datasets()`` (name -> numpy array, read on demand) and ``attrs`` of the
root group and of each dataset.
"""
import zlib

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


class _Reader:
    """Little-endian field access on the file's bytes."""

    def __init__(self, buf):
        self.b = buf
        self.so = 8  # size of offsets
        self.sl = 8  # size of lengths

    def uint(self, pos, n):
        return int.from_bytes(self.b[pos:pos + n], "little")

    def off(self, pos):
        return self.uint(pos, self.so)

    def length(self, pos):
        return self.uint(pos, self.sl)

    def sig(self, pos, expect):
        got = bytes(self.b[pos:pos + 4])
        if got != expect:
            raise ValueError(f"HDF5: expected {expect!r} at {pos:#x}, found {got!r}")


def _pad8(n):
    return (n + 7) & ~7


def _cstr(raw):
    return bytes(raw).split(b"\x00", 1)[0].decode("utf-8", "replace")


# ----------------------------------------------------------------- datatypes
class _Type:
    """A decoded datatype message: numpy dtype for numbers, or a string kind."""

    def __init__(self, kind, size, dtype=None, base=None, pad=0):
        self.kind = kind  # "num", "str", "vlstr", "vlseq", "other"
        self.size = size
        self.dtype = dtype
        self.base = base
        self.pad = pad


def _parse_type(r, pos):
    """Datatype message at pos -> (_Type, encoded length)."""
    cv = r.b[pos]
    cls, bits = cv & 0x0F, r.uint(pos + 1, 3)
    size = r.uint(pos + 4, 4)
    if cls == 0:  # fixed point
        order = ">" if bits & 1 else "<"
        return _Type("num", size, np.dtype(f"{order}{'i' if bits & 8 else 'u'}{size}")), 12
    if cls == 1:  # floating point
        order = ">" if bits & 1 else "<"
        if bits & 0x40 or size not in (2, 4, 8):
            raise NotImplementedError("HDF5: VAX or unusual floating-point layout")
        return _Type("num", size, np.dtype(f"{order}f{size}")), 20
    if cls == 3:  # fixed-length string
        return _Type("str", size, pad=bits & 0x0F), 8
    if cls == 9:  # variable length
        base, blen = _parse_type(r, pos + 8)
        if blen is None:  # e.g. netCDF's dimension lists: sequences of object references
            return _Type("other", size), None
        return _Type("vlstr" if (bits & 0x0F) == 1 else "vlseq", size, base=base), 8 + blen
    # compound (6), reference (7), enum (8), array (10), ...: not needed by SOFA data; their
    # encoded length is not tracked, so callers treat the value as unreadable
    return _Type("other", size), None


# --------------------------------------------------------------- dataspaces
def _parse_space(r, pos):
    ver, rank, flags = r.b[pos], r.b[pos + 1], r.b[pos + 2]
    if ver == 1:
        p = pos + 8
    elif ver == 2:
        if r.b[pos + 3] == 2:  # null dataspace
            return None
        p = pos + 4
    else:
        raise NotImplementedError(f"HDF5: dataspace version {ver}")
    return tuple(r.length(p + i * r.sl) for i in range(rank))


# ------------------------------------------------------------------- heaps
def _global_heap_object(r, addr, index, cache):
    """Object `index` of the global heap collection at addr (variable-length data)."""
    if addr not in cache:
        r.sig(addr, b"GCOL")
        size = r.length(addr + 8)
        objs, p, end = {}, addr + 8 + r.sl, addr + size
        while p + 8 + r.sl <= end:
            idx = r.uint(p, 2)
            if idx == 0:
                break
            n = r.length(p + 8)
            objs[idx] = bytes(r.b[p + 8 + r.sl:p + 8 + r.sl + n])
            p += 8 + r.sl + _pad8(n)
        cache[addr] = objs
    return cache[addr][index]


def _local_heap_data(r, addr):
    r.sig(addr, b"HEAP")
    return r.off(addr + 8 + 2 * r.sl)


class _FractalHeap:
    """Managed objects of a fractal heap (dense link and attribute storage)."""

    def __init__(self, r, addr):
        r.sig(addr, b"FRHP")
        self.r = r
        p = addr + 5
        self.id_len = r.uint(p, 2)
        self.filter_len = r.uint(p + 2, 2)
        self.flags = r.b[p + 4]
        self.max_obj = r.uint(p + 5, 4)
        p += 9 + r.sl + r.so + r.sl + r.so + 8 * r.sl  # ids, free space, managed/huge/tiny counters
        self.width = r.uint(p, 2)
        self.start = r.length(p + 2)
        self.max_direct = r.length(p + 2 + r.sl)
        self.max_bits = r.uint(p + 2 + 2 * r.sl, 2)
        p += 4 + 2 * r.sl + 2  # max heap size, starting rows
        self.root = r.off(p)
        self.rows = r.uint(p + r.so, 2)
        if self.filter_len:
            raise NotImplementedError("HDF5: filtered fractal heap")
        self.off_bytes = (self.max_bits + 7) // 8
        self.len_bytes = (min(self.max_direct, self.max_obj).bit_length() + 7) // 8
        self.blocks = []  # (block offset, address, size)
        if self.rows == 0:
            self._direct(self.root, self.start)
        else:
            self._indirect(self.root, self.rows)

    def _row_size(self, row):
        return self.start * (1 << max(row - 1, 0))

    def _direct(self, addr, size):
        r = self.r
        r.sig(addr, b"FHDB")
        self.blocks.append((r.uint(addr + 5 + r.so, self.off_bytes), addr, size))

    def _indirect(self, addr, nrows):
        r = self.r
        r.sig(addr, b"FHIB")
        p = addr + 5 + r.so + self.off_bytes
        for row in range(nrows):
            size = self._row_size(row)
            for _ in range(self.width):
                child = r.off(p)
                p += r.so
                if child == _UNDEF:
                    continue
                if size <= self.max_direct:
                    self._direct(child, size)
                else:
                    sub_rows = (size // (self.start * self.width)).bit_length()
                    self._indirect(child, sub_rows)

    def get(self, hid):
        kind = (hid[0] >> 4) & 3
        if kind == 2:  # tiny: data in the id itself
            return bytes(hid[1:1 + (hid[0] & 0x0F) + 1])
        if kind != 0:
            raise NotImplementedError("HDF5: huge fractal-heap objects")
        offset = int.from_bytes(hid[1:1 + self.off_bytes], "little")
        n = int.from_bytes(hid[1 + self.off_bytes:1 + self.off_bytes + self.len_bytes], "little")
        for bo, addr, size in self.blocks:
            if bo <= offset < bo + size:
                return bytes(self.r.b[addr + offset - bo:addr + offset - bo + n])
        raise ValueError("HDF5: fractal heap offset outside every direct block")


def _btree2_records(r, addr):
    """All records of a version-2 B-tree (depth 0 or 1)."""
    r.sig(addr, b"BTHD")
    node_size = r.uint(addr + 6, 4)
    rec_size = r.uint(addr + 10, 2)
    depth = r.uint(addr + 12, 2)
    root = r.off(addr + 16)
    nroot = r.uint(addr + 16 + r.so, 2)
    max_leaf = (node_size - 10) // rec_size
    nbytes = (max_leaf.bit_length() + 7) // 8

    def leaf(a, n):
        r.sig(a, b"BTLF")
        return [bytes(r.b[a + 6 + i * rec_size:a + 6 + (i + 1) * rec_size]) for i in range(n)]

    if depth == 0:
        return leaf(root, nroot)
    if depth != 1:
        raise NotImplementedError("HDF5: version-2 B-tree deeper than one level")
    r.sig(root, b"BTIN")
    recs = [bytes(r.b[root + 6 + i * rec_size:root + 6 + (i + 1) * rec_size]) for i in range(nroot)]
    p = root + 6 + nroot * rec_size
    out = []
    for i in range(nroot + 1):
        child, n = r.off(p), r.uint(p + r.so, nbytes)
        p += r.so + nbytes
        out += leaf(child, n)
        if i < nroot:
            out.append(recs[i])
    return out


# ----------------------------------------------------------- object headers
def _messages(r, addr):
    """(type, data position, size, flags) of every message of the object header at addr."""
    out = []
    if bytes(r.b[addr:addr + 4]) == b"OHDR":
        flags = r.b[addr + 5]
        p = addr + 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
        width = 1 << (flags & 3)
        size = r.uint(p, width)
        p += width
        blocks = [(p, p + size)]
        seen_blocks = set()
        hdr = 6 if flags & 0x04 else 4
        while blocks:
            p, end = blocks.pop(0)
            while p + hdr <= end:
                mtype, msize, mflags = r.b[p], r.uint(p + 1, 2), r.b[p + 3]
                d = p + hdr
                if mtype == 0x10:
                    c, n = r.off(d), r.length(d + r.so)
                    if c in seen_blocks or c + n > len(r.b):
                        raise ValueError(f"HDF5: bad continuation block at {c:#x}")
                    seen_blocks.add(c)
                    r.sig(c, b"OCHK")
                    blocks.append((c + 4, c + n - 4))
                elif mtype:
                    out.append((mtype, d, msize, mflags))
                p = d + msize
        return out
    if r.b[addr] != 1:
        raise NotImplementedError(f"HDF5: object header version {r.b[addr]}")
    nmsg, size = r.uint(addr + 2, 2), r.uint(addr + 8, 4)
    blocks = [(addr + 16, addr + 16 + size)]
    seen, seen_blocks = 0, set()
    while blocks and seen < nmsg:
        p, end = blocks.pop(0)
        while p + 8 <= end and seen < nmsg:
            mtype, msize, mflags = r.uint(p, 2), r.uint(p + 2, 2), r.b[p + 4]
            d = p + 8
            seen += 1
            if mtype == 0x10:
                c, n = r.off(d), r.length(d + r.so)
                if c in seen_blocks or c + n > len(r.b):
                    raise ValueError(f"HDF5: bad continuation block at {c:#x}")
                seen_blocks.add(c)
                blocks.append((c, c + n))
            elif mtype:
                out.append((mtype, d, msize, mflags))
            p = d + msize
    return out


def _parse_link(r, d):
    """Link message at d -> (name, object header address or None for soft/external links)."""
    flags = r.b[d + 1]
    p = d + 2
    ltype = 0
    if flags & 0x08:
        ltype = r.b[p]
        p += 1
    if flags & 0x04:
        p += 8
    if flags & 0x10:
        p += 1
    nlen_bytes = 1 << (flags & 3)
    nlen = r.uint(p, nlen_bytes)
    p += nlen_bytes
    name = bytes(r.b[p:p + nlen]).decode("utf-8")
    p += nlen
    return name, (r.off(p) if ltype == 0 else None)


class _Attr:
    """An attribute message at d of reader r (the file, or a fractal-heap object); fr is the file."""

    def __init__(self, r, d, fr, gheap):
        ver = r.b[d]
        nsz, tsz, ssz = r.uint(d + 2, 2), r.uint(d + 4, 2), r.uint(d + 6, 2)
        p = d + (9 if ver == 3 else 8)
        pad = _pad8 if ver == 1 else (lambda n: n)
        self.name = _cstr(r.b[p:p + nsz])
        p += pad(nsz)
        self.type, _ = _parse_type(r, p)
        p += pad(tsz)
        self.shape = _parse_space(r, p)
        p += pad(ssz)
        self._r, self._p, self._fr, self._gheap = r, p, fr, gheap

    def value(self):
        if self.shape is None or self.type.kind == "other":
            return None
        n = int(np.prod(self.shape)) if self.shape else 1
        raw = bytes(self._r.b[self._p:self._p + n * self.type.size])
        return _decode(self._fr, self.type, self.shape, raw, self._gheap)


def _decode(r, t, shape, raw, gheap):
    n = int(np.prod(shape)) if shape else 1
    if t.kind == "num":
        a = np.frombuffer(raw, dtype=t.dtype, count=n).astype(t.dtype.newbyteorder("="))
        return a.reshape(shape) if shape else a[0]
    if t.kind == "str":
        vals = [_cstr(raw[i * t.size:(i + 1) * t.size]).rstrip(" ") for i in range(n)]
    elif t.kind == "vlstr":
        vals = []
        for i in range(n):
            q = i * (4 + r.so + 4)
            ln = int.from_bytes(raw[q:q + 4], "little")
            addr = int.from_bytes(raw[q + 4:q + 4 + r.so], "little")
            idx = int.from_bytes(raw[q + 4 + r.so:q + 8 + r.so], "little")
            vals.append("" if ln == 0 or addr == 0 else
                        _global_heap_object(r, addr, idx, gheap)[:ln].decode("utf-8", "replace"))
    else:
        raise NotImplementedError(f"HDF5: datatype kind {t.kind}")
    if not shape:
        return vals[0]
    return np.array(vals, dtype=object).reshape(shape)


class Dataset:
    """A dataset: shape, type, attributes, and its data read on demand."""

    def __init__(self, f, name, msgs):
        r = f.r
        self._f, self.name = f, name
        self.shape, self.type, self.layout, self.filters = None, None, None, []
        self.attrs = {}
        for mtype, d, size, mflags in msgs:
            if mflags & 0x02 and mtype in (0x01, 0x03, 0x08, 0x0B):
                raise NotImplementedError(f"HDF5: shared message of type {mtype:#x} in '{name}'")
            if mtype == 0x01:
                self.shape = _parse_space(r, d)
            elif mtype == 0x03:
                self.type, _ = _parse_type(r, d)
            elif mtype == 0x08:
                self.layout = d
            elif mtype == 0x0B:
                self.filters = _parse_filters(r, d)
        self.attrs = f._attributes(msgs)

    def read(self):
        r, t = self._f.r, self.type
        if self.shape is None:
            return None
        shape = self.shape
        n = int(np.prod(shape)) if shape else 1
        nbytes = n * t.size
        d = self.layout
        ver, cls = r.b[d], r.b[d + 1]
        if ver < 3:
            raise NotImplementedError(f"HDF5: data layout version {ver}")
        if cls == 0:
            size = r.uint(d + 2, 2)
            raw = bytes(r.b[d + 4:d + 4 + size])
        elif cls == 1:
            addr = r.off(d + 2)
            raw = bytes(nbytes) if addr == _UNDEF else bytes(r.b[addr:addr + nbytes])
        elif cls == 2:
            raw = self._chunked(d, ver, shape, t.size)
        else:
            raise NotImplementedError(f"HDF5: layout class {cls}")
        return _decode(r, t, shape, raw, self._f._gheap)

    def _chunked(self, d, ver, shape, esize):
        r = self._f.r
        rank = len(shape)
        chunks = []  # (offsets, address, stored size, filter mask)
        if ver == 3:
            nd = r.b[d + 2]
            btree = r.off(d + 3)
            cdims = [r.uint(d + 3 + r.so + 4 * i, 4) for i in range(nd)]
            if btree != _UNDEF:
                self._btree1_chunks(btree, nd, chunks)
        else:
            flags, nd, enc = r.b[d + 2], r.b[d + 3], r.b[d + 4]
            cdims = [r.uint(d + 5 + enc * i, enc) for i in range(nd)]
            p = d + 5 + enc * nd
            itype = r.b[p]
            p += 1
            if itype == 1:  # single chunk
                size, mask = None, 0
                if flags & 0x02:
                    size, mask = r.length(p), r.uint(p + r.sl, 4)
                    p += r.sl + 4
                addr = r.off(p)
                if addr != _UNDEF:
                    chunks.append(((0,) * rank, addr, size, mask))
            elif itype == 2:  # implicit: chunks stored in order, unfiltered
                addr = r.off(p)
                grid = [-(-shape[i] // cdims[i]) for i in range(rank)]
                csize = int(np.prod(cdims[:rank])) * esize
                for k, idx in enumerate(np.ndindex(*grid)):
                    chunks.append((tuple(i * c for i, c in zip(idx, cdims)), addr + k * csize, csize, 0))
            elif itype == 3:  # fixed array
                self._fixed_array_chunks(r.off(p + 1), shape, cdims, chunks)
            else:
                raise NotImplementedError(f"HDF5: chunk index type {itype}")
        cdims = cdims[:rank]
        out = np.zeros(shape, dtype=np.dtype((np.void, esize))) if rank else None
        csize = int(np.prod(cdims)) * esize
        for offs, addr, size, mask in chunks:
            raw = bytes(r.b[addr:addr + (size if size is not None else csize)])
            raw = _unfilter(raw, self.filters, mask, esize)
            if len(raw) < csize:
                raise ValueError(f"HDF5: chunk of '{self.name}' is {len(raw)} bytes, expected {csize}")
            block = np.frombuffer(raw[:csize], dtype=out.dtype).reshape(cdims)
            dst = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
            src = tuple(slice(0, sl.stop - sl.start) for sl in dst)
            out[dst] = block[src]
        return out.tobytes()

    def _btree1_chunks(self, addr, nd, chunks, parent_level=None):
        r = self._f.r
        r.sig(addr, b"TREE")
        level, used = r.b[addr + 5], r.uint(addr + 6, 2)
        if parent_level is not None and level >= parent_level:
            raise ValueError("HDF5: chunk B-tree levels do not decrease")
        p = addr + 8 + 2 * r.so
        ksize = 8 + 8 * nd
        for i in range(used):
            size, mask = r.uint(p, 4), r.uint(p + 4, 4)
            offs = tuple(r.uint(p + 8 + 8 * k, 8) for k in range(nd - 1))
            child = r.off(p + ksize)
            if level == 0:
                chunks.append((offs, child, size, mask))
            else:
                self._btree1_chunks(child, nd, chunks, level)
            p += ksize + r.so

    def _fixed_array_chunks(self, addr, shape, cdims, chunks):
        r = self._f.r
        r.sig(addr, b"FAHD")
        client, esz, page_bits = r.b[addr + 5], r.b[addr + 6], r.b[addr + 7]
        nent = r.length(addr + 8)
        dblock = r.off(addr + 8 + r.sl)
        if nent > (1 << page_bits):
            raise NotImplementedError("HDF5: paged fixed-array chunk index")
        r.sig(dblock, b"FADB")
        p = dblock + 6 + r.so
        rank = len(shape)
        grid = [-(-shape[i] // cdims[i]) for i in range(rank)]
        for k, idx in enumerate(np.ndindex(*grid)):
            if k >= nent:
                break
            q = p + k * esz
            addr_k = r.off(q)
            if client == 1:  # filtered: address, chunk size, filter mask
                size = r.uint(q + r.so, esz - r.so - 4)
                mask = r.uint(q + esz - 4, 4)
            else:
                size, mask = None, 0
            if addr_k != _UNDEF:
                chunks.append((tuple(i * c for i, c in zip(idx, cdims)), addr_k, size, mask))


def _parse_filters(r, d):
    ver, n = r.b[d], r.b[d + 1]
    p = d + (8 if ver == 1 else 2)
    out = []
    for _ in range(n):
        fid = r.uint(p, 2)
        if ver == 1 or fid >= 256:
            nlen = r.uint(p + 2, 2)
            p += 4
        else:
            nlen = 0
            p += 2
        ncd = r.uint(p + 2, 2)
        p += 4
        p += _pad8(nlen) if ver == 1 else nlen
        cd = [r.uint(p + 4 * i, 4) for i in range(ncd)]
        p += 4 * ncd
        if ver == 1 and ncd % 2:
            p += 4
        out.append((fid, cd))
    return out


def _unfilter(raw, filters, mask, esize):
    """Undo the filter pipeline (applied in order on write, so undone in reverse)."""
    for k in range(len(filters) - 1, -1, -1):
        if mask & (1 << k):
            continue
        fid, _ = filters[k]
        if fid == 1:
            raw = zlib.decompress(raw)
        elif fid == 2:
            a = np.frombuffer(raw, dtype=np.uint8)
            m = a.size // esize
            body = a[:m * esize].reshape(esize, m).T.reshape(-1)
            raw = body.tobytes() + a[m * esize:].tobytes()
        elif fid == 3:
            raw = raw[:-4]
        else:
            raise NotImplementedError(f"HDF5: filter {fid}")
    return raw


class File:
    """An HDF5 file held in memory: root attributes and the datasets of the root group."""

    def __init__(self, path):
        with open(path, "rb") as fh:
            buf = fh.read()
        if buf[:8] != _SIG:
            raise ValueError(f"{path}: not an HDF5 file")
        r = _Reader(memoryview(buf))
        ver = buf[8]
        if ver in (0, 1):
            r.so, r.sl = buf[13], buf[14]
            p = 24 + (4 if ver == 1 else 0) + 4 * r.so
            root = r.off(p + r.so)
        elif ver in (2, 3):
            r.so, r.sl = buf[9], buf[10]
            root = r.off(12 + 3 * r.so)
        else:
            raise NotImplementedError(f"HDF5: superblock version {ver}")
        self.r = r
        self._gheap = {}
        msgs = _messages(r, root)
        self.attrs = self._attributes(msgs)
        self._links = self._group_links(msgs)

    def _attributes(self, msgs):
        r = self.r
        out = {}
        for mtype, d, size, mflags in msgs:
            if mtype == 0x0C:
                a = _Attr(r, d, r, self._gheap)
                out[a.name] = a
            elif mtype == 0x15:  # attribute info: dense storage
                flags = r.b[d + 1]
                p = d + 2 + (2 if flags & 1 else 0)
                heap_addr, name_bt = r.off(p), r.off(p + r.so)
                if heap_addr == _UNDEF:
                    continue
                heap = _FractalHeap(r, heap_addr)
                for rec in _btree2_records(r, name_bt):
                    blob = heap.get(rec[:heap.id_len])
                    tmp = _Reader(memoryview(blob))
                    tmp.so, tmp.sl = r.so, r.sl
                    a = _Attr(tmp, 0, r, self._gheap)
                    out[a.name] = a
        return out

    def _group_links(self, msgs):
        r = self.r
        links = {}
        for mtype, d, size, mflags in msgs:
            if mtype == 0x06:
                name, addr = _parse_link(r, d)
                if addr is not None:
                    links[name] = addr
            elif mtype == 0x02:
                flags = r.b[d + 1]
                p = d + 2 + (8 if flags & 1 else 0)
                heap_addr, name_bt = r.off(p), r.off(p + r.so)
                if heap_addr == _UNDEF:
                    continue
                heap = _FractalHeap(r, heap_addr)
                for rec in _btree2_records(r, name_bt):
                    blob = heap.get(rec[4:4 + heap.id_len])
                    tmp = _Reader(memoryview(blob))
                    tmp.so, tmp.sl = r.so, r.sl
                    name, addr = _parse_link(tmp, 0)
                    if addr is not None:
                        links[name] = addr
            elif mtype == 0x11:
                self._symbol_table(r.off(d), _local_heap_data(r, r.off(d + r.so)), links)
        return links

    def _symbol_table(self, addr, heap_data, links, parent_level=None):
        r = self.r
        r.sig(addr, b"TREE")
        level, used = r.b[addr + 5], r.uint(addr + 6, 2)
        if parent_level is not None and level >= parent_level:
            raise ValueError("HDF5: group B-tree levels do not decrease")
        p = addr + 8 + 2 * r.so + r.sl
        for _ in range(used):
            child = r.off(p)
            if level > 0:
                self._symbol_table(child, heap_data, links, level)
            else:
                r.sig(child, b"SNOD")
                n = r.uint(child + 6, 2)
                e = child + 8
                for _ in range(n):
                    name = _cstr(r.b[heap_data + r.off(e):heap_data + r.off(e) + 256])
                    links[name] = r.off(e + r.so)
                    e += 2 * r.so + 24
            p += r.so + r.sl

    def datasets(self):
        """Datasets of the root group, keyed by their HDF5 names (groups are left out)."""
        out = {}
        for name, addr in self._links.items():
            msgs = _messages(self.r, addr)
            if any(m[0] == 0x08 for m in msgs):
                out[name] = Dataset(self, name, msgs)
        return out
