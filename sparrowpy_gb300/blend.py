"""Meshes from Blender .blend files, read without Blender.

sparrowpy reads a .blend file with Blender's own Python modules
(utils/blender.py:22-97: bpy.ops.wm.open_mainfile, then the mesh of the
object named "Geometry" through bmesh).  Blender is not installed here, so
this module reads the file format itself:

* the header: "BLENDER", the pointer size ('_' 4 bytes, '-' 8 bytes), the
  byte order ('v' little, 'V' big) and the version;
* the file blocks: a code, the data length, the block's old memory address,
  its struct (SDNA index) and the number of structs, then the data;
* the DNA1 block: the struct catalogue (names, types, type lengths and the
  fields of every struct), through which every other block is decoded.

A mesh is read in the layout of the file's version: Blender 2.8-3.4 keep
vertices as MVert structs and faces as MPoly/MLoop structs; Blender 3.5
and later keep a "position" float3 layer, face offsets
(poly_offset_indices / face_offset_indices) and a ".corner_vert" layer.
Only the mesh data block is read (the object's transform and modifiers are
not applied, as bmesh.from_mesh does not apply them).
"""
import re

import numpy as np


class BlendFile:
    """The blocks and the struct catalogue of a .blend file."""

    def __init__(self, path):
        with open(path, "rb") as fh:
            self.buf = fh.read()
        b = self.buf
        if b[:7] != b"BLENDER":
            raise ValueError(f"{path}: not a .blend file (compressed files must be decompressed first)")
        if b[7:8] not in (b"_", b"-") or b[8:9] not in (b"v", b"V"):
            raise NotImplementedError(f"{path}: .blend header {b[:17]!r} is not supported")
        self.ptr = 4 if b[7:8] == b"_" else 8
        self.end = "<" if b[8:9] == b"v" else ">"
        self.version = int(b[9:12])
        self.blocks = []  # (code, length, old address, sdna index, count, data offset)
        p = 12
        head = 16 + self.ptr
        while p + head <= len(b):
            code = b[p:p + 4]
            length, = np.frombuffer(b, self.end + "i4", 1, p + 4)
            old = int(np.frombuffer(b, self.end + ("u8" if self.ptr == 8 else "u4"), 1, p + 8)[0])
            sdna, count = np.frombuffer(b, self.end + "i4", 2, p + 8 + self.ptr)
            if length < 0 or p + head + int(length) > len(b):
                raise ValueError(f"{path}: block at {p} runs past the end of the file")
            self.blocks.append((code, int(length), old, int(sdna), int(count), p + head))
            if code == b"ENDB":
                break
            p += head + int(length)
        self.by_old = {blk[2]: blk for blk in self.blocks if blk[0] != b"ENDB"}
        dna = [blk for blk in self.blocks if blk[0] == b"DNA1"]
        if not dna:
            raise ValueError(f"{path}: no DNA1 block")
        self._parse_dna(dna[0][5])

    # -------------------------------------------------------------- SDNA
    def _parse_dna(self, p):
        b, e = self.buf, self.end

        def i32(q):
            return int(np.frombuffer(b, e + "i4", 1, q)[0])

        def strings(q, n):
            out = []
            for _ in range(n):
                z = b.index(b"\x00", q)
                out.append(b[q:z].decode("ascii"))
                q = z + 1
            return out, q

        def align4(q):
            return (q + 3) & ~3

        assert b[p:p + 4] == b"SDNA" and b[p + 4:p + 8] == b"NAME"
        names, q = strings(p + 12, i32(p + 8))
        q = align4(q)
        assert b[q:q + 4] == b"TYPE"
        types, q = strings(q + 8, i32(q + 4))
        q = align4(q)
        assert b[q:q + 4] == b"TLEN"
        tlen = np.frombuffer(b, e + "i2", len(types), q + 4).astype(int)
        q = align4(q + 4 + 2 * len(types))
        assert b[q:q + 4] == b"STRC"
        n_structs = i32(q + 4)
        q += 8
        self.structs = []      # per SDNA index: (type name, [(field type, field name)])
        for _ in range(n_structs):
            t, nf = np.frombuffer(b, e + "i2", 2, q)
            fields = np.frombuffer(b, e + "i2", 2 * int(nf), q + 4).reshape(-1, 2)
            self.structs.append((types[int(t)], [(types[int(ft)], names[int(fn)]) for ft, fn in fields]))
            q += 4 + 4 * int(nf)
        self.tlen = dict(zip(types, tlen))
        self.struct_index = {name: i for i, (name, _) in enumerate(self.structs)}
        self._layouts = {}

    def layout(self, type_name):
        """Fields of a struct: name -> (offset, type, is pointer, array dims)."""
        if type_name not in self._layouts:
            out, off = {}, 0
            for ftype, fname in self.structs[self.struct_index[type_name]][1]:
                is_ptr = fname.startswith("*") or fname.startswith("(*")
                dims = tuple(int(d) for d in re.findall(r"\[(\d+)\]", fname))
                base = re.sub(r"[\*\(\)\[\]0-9]", "", fname.split("[")[0]).strip()
                if fname.startswith("(*"):
                    base = re.sub(r"[\*\(\)]", "", fname.split(")")[0])
                size = (self.ptr if is_ptr else int(self.tlen[ftype])) * int(np.prod(dims) if dims else 1)
                out[base] = (off, ftype, is_ptr, dims)
                off += size
            self._layouts[type_name] = out
        return self._layouts[type_name]

    def field(self, type_name, base, name):
        """Value of a scalar field, pointer (old address), char array (string) or nested struct offset."""
        path = name.split(".")
        for k, part in enumerate(path):
            off, ftype, is_ptr, dims = self.layout(type_name)[part]
            base += off
            if k < len(path) - 1:
                type_name = ftype
        if is_ptr:
            return int(np.frombuffer(self.buf, self.end + ("u8" if self.ptr == 8 else "u4"), 1, base)[0])
        if ftype == "char" and dims:
            raw = self.buf[base:base + int(np.prod(dims))]
            return raw.split(b"\x00", 1)[0].decode("utf-8", "replace")
        if ftype in self.struct_index:
            return base
        dt = {"int": "i4", "uint": "u4", "short": "i2", "ushort": "u2", "float": "f4", "double": "f8",
              "char": "u1", "uchar": "u1", "int8_t": "i1", "int64_t": "i8", "uint64_t": "u8"}[ftype]
        n = int(np.prod(dims)) if dims else 1
        v = np.frombuffer(self.buf, self.end + dt, n, base)
        return v.reshape(dims) if dims else v[0].item()

    def has(self, type_name, name):
        return name in self.layout(type_name)

    def data_of(self, old):
        """(offset, length, struct type name, count) of the block an old address points to."""
        blk = self.by_old.get(old)
        if blk is None:
            raise ValueError(f"no block at old address {old:#x}")
        return blk[5], blk[1], self.structs[blk[3]][0], blk[4]

    def blocks_of(self, type_name):
        idx = self.struct_index.get(type_name)
        return [blk for blk in self.blocks if blk[3] == idx and blk[0] not in (b"DNA1", b"ENDB")]


def _layer(f, cdata_base, type_code=None, name=None):
    """Data offset and element count of a CustomData layer chosen by type code or name."""
    layers = f.field("CustomData", cdata_base, "layers")
    n = f.field("CustomData", cdata_base, "totlayer")
    if not layers or n <= 0:
        return None
    off, _, _, _ = f.data_of(layers)
    size = int(f.tlen["CustomDataLayer"])
    for i in range(n):
        base = off + i * size
        if (type_code is not None and f.field("CustomDataLayer", base, "type") == type_code) or \
                (name is not None and f.field("CustomDataLayer", base, "name") == name):
            data = f.field("CustomDataLayer", base, "data")
            if data:
                return f.data_of(data)
    return None


def read_mesh(path, object_name="Geometry"):
    """Vertices (n, 3) and faces (lists of vertex indices) of the named object's mesh."""
    f = BlendFile(path)
    mesh_old = None
    for blk in f.blocks_of("Object"):
        if f.field("Object", blk[5], "id.name")[2:] == object_name:
            mesh_old = f.field("Object", blk[5], "data")
            break
    if mesh_old is None:
        raise ValueError(f"{path}: no object named '{object_name}'")
    mbase, _, stype, _ = f.data_of(mesh_old)
    if stype != "Mesh":
        raise ValueError(f"{path}: object '{object_name}' holds a {stype}, not a mesh")
    e = f.end
    n_vert = f.field("Mesh", mbase, "totvert")
    n_face = f.field("Mesh", mbase, "faces_num" if f.has("Mesh", "faces_num") else "totpoly")
    n_loop = f.field("Mesh", mbase, "totloop")
    vdata = f.field("Mesh", mbase, "vdata")
    ldata = f.field("Mesh", mbase, "ldata")
    pos = _layer(f, vdata, name="position")
    if pos is not None:  # Blender 3.5 and later: generic attributes
        verts = np.frombuffer(f.buf, e + "f4", 3 * n_vert, pos[0]).reshape(n_vert, 3)
    else:  # MVert structs (CD_MVERT = 0)
        mv = _layer(f, vdata, type_code=0)
        if mv is None:
            raise NotImplementedError(f"{path}: no vertex positions found in the mesh")
        co, _, _, _ = f.layout("MVert")["co"]
        stride = int(f.tlen["MVert"])
        raw = np.frombuffer(f.buf, np.uint8, stride * n_vert, mv[0]).reshape(n_vert, stride)
        verts = raw[:, co:co + 12].copy().view(e + "f4").reshape(n_vert, 3)
    off_name = "face_offset_indices" if f.has("Mesh", "face_offset_indices") else "poly_offset_indices"
    if f.has("Mesh", off_name) and f.field("Mesh", mbase, off_name):
        offsets = np.frombuffer(f.buf, e + "i4", n_face + 1, f.data_of(f.field("Mesh", mbase, off_name))[0])
        cv = _layer(f, ldata, name=".corner_vert")
        if cv is None:
            raise NotImplementedError(f"{path}: no corner vertices found in the mesh")
        corner = np.frombuffer(f.buf, e + "i4", n_loop, cv[0])
        faces = [corner[offsets[i]:offsets[i + 1]].astype(int).tolist() for i in range(n_face)]
    else:  # MPoly (CD_MPOLY = 25) and MLoop (CD_MLOOP = 26) structs
        mp, ml = _layer(f, f.field("Mesh", mbase, "pdata"), type_code=25), _layer(f, ldata, type_code=26)
        if mp is None or ml is None:
            raise NotImplementedError(f"{path}: no faces found in the mesh")
        ps, ls = int(f.tlen["MPoly"]), int(f.tlen["MLoop"])
        lv = np.array([f.field("MLoop", ml[0] + i * ls, "v") for i in range(n_loop)], dtype=int)
        faces = []
        for i in range(n_face):
            start = f.field("MPoly", mp[0] + i * ps, "loopstart")
            count = f.field("MPoly", mp[0] + i * ps, "totloop")
            faces.append(lv[start:start + count].tolist())
    return verts.astype(np.float64), faces
