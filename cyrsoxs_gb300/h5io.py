"""HDF5 subset reader and writer for the CyRSoXS on-disk formats, without
libhdf5 (neither h5py nor libhdf5 is part of this stack).

Covered (from the published HDF5 file format specification):
* reading files with a version 0 or 1 superblock, version 1 object headers
  (with continuation blocks), symbol-table groups (v1 B-tree of symbol nodes
  plus a local heap), dataspace messages v1/v2, fixed-point and IEEE float
  datatypes, contiguous, compact and chunked (v1 B-tree index, deflate and
  shuffle filters) layouts, and attributes whose values are numbers or
  variable-length strings in a global heap (the DIMENSION_LABELS that record
  whether a morphology is stored ZYX or XYZ);
* writing files of the same family: contiguous little-endian datasets,
  symbol-table groups, and DIMENSION_LABELS attributes.

The CyRSoXS layouts:
* morphology (include/Input/readH5.h:45-539, docs/DATA.md): groups
  ``Euler_Angles`` (Mat_i_Vfrac, Mat_i_S, Mat_i_Theta, Mat_i_Psi) or
  ``Vector_Morphology`` (Mat_i_alignment [.., 3], Mat_i_unaligned), and
  ``Morphology_Parameters`` (PhysSize, NumMaterial);
* scattering patterns (include/utils.h:38-87, include/Output/writeH5.h:40-68):
  ``<dir>/Energy_<E:.2f>.h5`` with ``KIDList/KVec`` [k][3] and
  ``K<k>/projection`` [Ny][Nx] labelled (Qy, Qx);
* polarization (writeH5.h:77-110): ``Polarization/Polarization{X,Y,Z}.h5``
  with dataset ``p{X,Y,Z}`` [Z][Y][X][2];
* morphology dump (writeH5.h:117-170): ``Material_<m>/{S,Theta,Psi,Vfrac}``
  (Euler) or ``{Sx,Sy,Sz,UnalignedFraction}`` (vector).
"""
from __future__ import annotations

import os
import struct
import zlib
from dataclasses import dataclass

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


# ---------------------------------------------------------------------------
# reader
# ---------------------------------------------------------------------------
class _Reader:
    def __init__(self, data: bytes):
        self.d = data
        if data[:8] != SIGNATURE:
            raise ValueError("not an HDF5 file (signature)")
        ver = data[8]
        if ver not in (0, 1):
            raise ValueError(f"HDF5 superblock version {ver} is not supported (0 and 1 are)")
        self.so, self.sl = data[13], data[14]
        if self.so != 8 or self.sl != 8:
            raise ValueError("only 8-byte offsets and lengths are supported")
        pos = 24 if ver == 0 else 28
        self.base = self.u(pos, 8)
        pos += 32  # base, free-space, end-of-file and driver-info addresses
        self.root = self._symbol_entry(pos)
        self._gheap = {}

    def u(self, pos, n):
        return int.from_bytes(self.d[pos:pos + n], "little")

    def _symbol_entry(self, pos):
        name_off, header = self.u(pos, 8), self.u(pos + 8, 8)
        cache = self.u(pos + 16, 4)
        scratch = (self.u(pos + 24, 8), self.u(pos + 32, 8)) if cache == 1 else None
        return name_off, header, scratch

    # object headers --------------------------------------------------------
    def messages(self, addr):
        d = self.d
        if d[addr] == 1:
            nmsg = self.u(addr + 2, 2)
            size = self.u(addr + 8, 4)
            blocks = [(addr + 16, size)]
            out = []
            while blocks and len(out) < nmsg:
                pos, length = blocks.pop(0)
                end = pos + length
                while pos + 8 <= end and len(out) < nmsg:
                    mtype, msize, flags = self.u(pos, 2), self.u(pos + 2, 2), d[pos + 4]
                    body = d[pos + 8:pos + 8 + msize]
                    if mtype == 0x10:  # continuation
                        blocks.append((int.from_bytes(body[0:8], "little"), int.from_bytes(body[8:16], "little")))
                    out.append((mtype, flags, body))
                    pos += 8 + msize
            return out
        raise ValueError("only version 1 object headers are supported")

    # groups ------------------------------------------------------------------
    def _heap_data(self, heap):
        if self.d[heap:heap + 4] != b"HEAP":
            raise ValueError("bad local heap")
        return self.u(heap + 24, 8)

    def _heap_name(self, heap_data, off):
        end = self.d.index(b"\0", heap_data + off)
        return self.d[heap_data + off:end].decode()

    def group_members(self, header_addr, scratch=None):
        btree = heap = None
        for mtype, _, body in self.messages(header_addr):
            if mtype == 0x11:
                btree, heap = int.from_bytes(body[0:8], "little"), int.from_bytes(body[8:16], "little")
        if btree is None and scratch:
            btree, heap = scratch
        if btree is None:
            raise ValueError("group without a symbol table (only symbol-table groups are supported)")
        hdata = self._heap_data(heap)
        out = {}
        self._walk_group_tree(btree, hdata, out)
        return out

    def _walk_group_tree(self, node, hdata, out):
        d = self.d
        if d[node:node + 4] != b"TREE":
            raise ValueError("bad group B-tree node")
        level, used = d[node + 5], self.u(node + 6, 2)
        pos = node + 24 + 8  # first key
        for _ in range(used):
            child = self.u(pos, 8)
            pos += 16
            if level > 0:
                self._walk_group_tree(child, hdata, out)
            else:
                if d[child:child + 4] != b"SNOD":
                    raise ValueError("bad symbol node")
                n = self.u(child + 6, 2)
                for i in range(n):
                    e = child + 8 + 40 * i
                    name_off, header, scratch = self._symbol_entry(e)
                    out[self._heap_name(hdata, name_off)] = (header, scratch)

    # datatypes, dataspaces, attributes --------------------------------------------
    @staticmethod
    def _dtype(body):
        cls, bits, size = body[0] & 0x0F, body[1] | (body[2] << 8) | (body[3] << 16), int.from_bytes(body[4:8], "little")
        if cls == 0:  # fixed point
            end = ">" if bits & 1 else "<"
            return np.dtype(f"{end}{'i' if bits & 8 else 'u'}{size}"), 8 + 4
        if cls == 1:  # IEEE float
            end = ">" if bits & 1 else "<"
            return np.dtype(f"{end}f{size}"), 8 + 12
        if cls == 9:  # variable length
            return ("vlen-string" if (bits & 0xF) == 1 else "vlen"), None
        if cls == 3:  # fixed-length string
            return np.dtype(f"S{size}"), 8
        raise ValueError(f"HDF5 datatype class {cls} is not supported")

    def _dataspace(self, body):
        ver, ndim, flags = body[0], body[1], body[2]
        pos = 8 if ver == 1 else 4
        if ver == 2 and body[3] == 0:  # scalar
            return ()
        dims = tuple(int.from_bytes(body[pos + 8 * i:pos + 8 * i + 8], "little") for i in range(ndim))
        return dims

    def _gheap_object(self, coll, index):
        if coll not in self._gheap:
            d = self.d
            if d[coll:coll + 4] != b"GCOL":
                raise ValueError("bad global heap collection")
            size = self.u(coll + 8, 8)
            pos, end, objs = coll + 16, coll + size, {}
            while pos + 16 <= end:
                idx, osize = self.u(pos, 2), self.u(pos + 8, 8)
                if idx == 0:
                    break
                objs[idx] = d[pos + 16:pos + 16 + osize]
                pos += 16 + ((osize + 7) & ~7)
            self._gheap[coll] = objs
        return self._gheap[coll][index]

    def attributes(self, header_addr):
        out = {}
        for mtype, _, body in self.messages(header_addr):
            if mtype != 0x0C:
                continue
            ver = body[0]
            nlen, tlen, slen = (int.from_bytes(body[2 + 2 * i:4 + 2 * i], "little") for i in range(3))
            pad = (lambda n: (n + 7) & ~7) if ver == 1 else (lambda n: n)
            pos = 8 if ver in (1, 2) else 9
            name = body[pos:pos + nlen].split(b"\0")[0].decode()
            pos += pad(nlen)
            dt, _ = self._dtype(body[pos:pos + tlen])
            pos += pad(tlen)
            dims = self._dataspace(body[pos:pos + slen])
            pos += pad(slen)
            count = int(np.prod(dims)) if dims else 1
            raw = body[pos:]
            if dt == "vlen-string":
                vals = []
                for i in range(count):
                    e = raw[16 * i:16 * i + 16]
                    n, coll, idx = (int.from_bytes(e[0:4], "little"), int.from_bytes(e[4:12], "little"),
                                    int.from_bytes(e[12:16], "little"))
                    vals.append(self._gheap_object(coll, idx)[:n].split(b"\0")[0].decode() if coll else "")
                out[name] = vals
            elif isinstance(dt, np.dtype):
                out[name] = np.frombuffer(raw[:count * dt.itemsize], dt).reshape(dims or ())
        return out

    # datasets ------------------------------------------------------------------
    def dataset(self, header_addr) -> np.ndarray:
        dtype = dims = layout = None
        filters = []
        for mtype, _, body in self.messages(header_addr):
            if mtype == 0x01:
                dims = self._dataspace(body)
            elif mtype == 0x03:
                dtype, _ = self._dtype(body)
            elif mtype == 0x08:
                layout = body
            elif mtype == 0x0B:
                filters = self._filters(body)
        if dtype is None or dims is None or layout is None or not isinstance(dtype, np.dtype):
            raise ValueError("unsupported dataset (no numeric type, space or layout)")
        count = int(np.prod(dims)) if dims else 1
        ver = layout[0]
        if ver != 3:
            raise ValueError(f"data layout message version {ver} is not supported (3 is)")
        cls = layout[1]
        if cls == 0:  # compact
            size = int.from_bytes(layout[2:4], "little")
            raw = layout[4:4 + size]
        elif cls == 1:  # contiguous
            addr = int.from_bytes(layout[2:10], "little")
            if addr == UNDEF:
                return np.zeros(dims, dtype.newbyteorder("="))
            raw = self.d[addr:addr + count * dtype.itemsize]
        elif cls == 2:  # chunked, v1 B-tree index
            nd = layout[2]
            addr = int.from_bytes(layout[3:11], "little")
            cdims = [int.from_bytes(layout[11 + 4 * i:15 + 4 * i], "little") for i in range(nd)][:-1]
            return self._chunked(addr, dims, cdims, dtype, filters)
        else:
            raise ValueError(f"layout class {cls} is not supported")
        return np.frombuffer(raw, dtype).reshape(dims).astype(dtype.newbyteorder("="))

    @staticmethod
    def _filters(body):
        ver, n = body[0], body[1]
        pos = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = int.from_bytes(body[pos:pos + 2], "little")
            if ver == 1 or fid >= 256:
                nlen = int.from_bytes(body[pos + 2:pos + 4], "little")
                ncv = int.from_bytes(body[pos + 6:pos + 8], "little")
                pos += 8 + ((nlen + 7) & ~7 if ver == 1 else nlen)
            else:
                ncv = int.from_bytes(body[pos + 6:pos + 8], "little")
                pos += 8
            cvals = [int.from_bytes(body[pos + 4 * i:pos + 4 * i + 4], "little") for i in range(ncv)]
            pos += 4 * ncv + (4 if ver == 1 and ncv % 2 else 0)
            out.append((fid, cvals))
        return out

    def _chunked(self, addr, dims, cdims, dtype, filters):
        out = np.zeros(dims, dtype.newbyteorder("="))
        nd = len(dims)
        for offs, raw, mask in self._chunks(addr, nd):
            for j, (fid, cv) in enumerate(reversed(filters)):
                if mask & (1 << (len(filters) - 1 - j)):
                    continue
                if fid == 1:
                    raw = zlib.decompress(raw)
                elif fid == 2:  # shuffle
                    es = cv[0] if cv else dtype.itemsize
                    a = np.frombuffer(raw, np.uint8)
                    raw = a.reshape(es, -1).T.tobytes()
                else:
                    raise ValueError(f"HDF5 filter {fid} is not supported (deflate and shuffle are)")
            chunk = np.frombuffer(raw, dtype)[: int(np.prod(cdims))].reshape(cdims)
            sl = tuple(slice(o, min(o + c, n)) for o, c, n in zip(offs, cdims, dims))
            out[sl] = chunk[tuple(slice(0, s.stop - s.start) for s in sl)]
        return out

    def _chunks(self, node, nd):
        d = self.d
        if d[node:node + 4] != b"TREE" or d[node + 4] != 1:
            raise ValueError("bad chunk B-tree node")
        level, used = d[node + 5], self.u(node + 6, 2)
        ksize = 8 + 8 * (nd + 1)
        pos = node + 24
        for _ in range(used):
            csize, mask = self.u(pos, 4), self.u(pos + 4, 4)
            offs = [self.u(pos + 8 + 8 * i, 8) for i in range(nd)]
            child = self.u(pos + ksize, 8)
            if level > 0:
                yield from self._chunks(child, nd)
            else:
                yield offs, d[child:child + csize], mask
            pos += ksize + 8

    # paths ---------------------------------------------------------------------------
    def lookup(self, path):
        header, scratch = self.root[1], self.root[2]
        for part in [p for p in path.split("/") if p]:
            members = self.group_members(header, scratch)
            if part not in members:
                raise KeyError(f"{path}: '{part}' not found")
            header, scratch = members[part]
        return header


class File:
    """Read-only view of an HDF5 file of the supported subset."""

    def __init__(self, path: str):
        with open(path, "rb") as f:
            self._r = _Reader(f.read())

    def exists(self, path: str) -> bool:
        try:
            self._r.lookup(path)
            return True
        except KeyError:
            return False

    def keys(self, path: str = "/"):
        header = self._r.lookup(path)
        scratch = self._r.root[2] if path.strip("/") == "" else None
        return sorted(self._r.group_members(header, scratch))

    def read(self, path: str) -> np.ndarray:
        return self._r.dataset(self._r.lookup(path))

    def attrs(self, path: str) -> dict:
        return self._r.attributes(self._r.lookup(path))

    def labels(self, path: str):
        a = self.attrs(path).get("DIMENSION_LABELS")
        return list(a) if a is not None else None


# ---------------------------------------------------------------------------
# morphology reading (include/Input/readH5.h)
# ---------------------------------------------------------------------------
@dataclass
class Morphology:
    num_material: int
    phys_size: float
    order: int            # MorphologyOrder: 0 ZYX, 1 XYZ (include/Datatypes.h:170-177)
    dims_xyz: tuple       # (X, Y, Z)
    voxels: np.ndarray    # float32 [M][Z][Y][X][4], Voxel::s1 per material


def _to_zyx(a, order, comps):
    if order == 1:  # XYZ: stored [X][Y][Z](...)
        axes = (2, 1, 0) + ((3,) if comps > 1 else ())
        return np.ascontiguousarray(np.transpose(a, axes))
    return a


def read_morphology(path: str, morphology_type: int) -> Morphology:
    """Reads an Euler (morphology_type 0) or vector (1) morphology as the
    reference does: the order comes from the labels of the first scalar
    dataset (Z..X = ZYX, X..Z = XYZ), Euler S absent means unaligned, and
    theta, psi are zeroed where S = 0 (readH5.h:484-531)."""
    f = File(path)
    if not f.exists("Morphology_Parameters/NumMaterial"):
        raise KeyError("Morphology_Parameters/NumMaterial not found")
    nmat = int(np.asarray(f.read("Morphology_Parameters/NumMaterial")).reshape(-1)[0])
    phys = float(np.asarray(f.read("Morphology_Parameters/PhysSize")).reshape(-1)[0])
    group, first = ("Euler_Angles", "Mat_1_Vfrac") if morphology_type == 0 else ("Vector_Morphology", "Mat_1_unaligned")
    ref = f.read(f"{group}/{first}")
    if ref.ndim != 3:
        raise ValueError(f"expected a 3D array for {first}, found {ref.ndim}D")
    lab = f.labels(f"{group}/{first}") or []
    if len(lab) >= 3 and lab[0] == "Z" and lab[2] == "X":
        order, (Z, Y, X) = 0, ref.shape
    elif len(lab) >= 3 and lab[0] == "X" and lab[2] == "Z":
        order, (X, Y, Z) = 1, ref.shape
    else:
        raise ValueError("only XYZ/ZYX ordering supported (DIMENSION_LABELS)")
    vox = np.zeros((nmat, Z, Y, X, 4), np.float32)
    for m in range(1, nmat + 1):
        if morphology_type == 0:
            vox[m - 1, ..., 3] = _to_zyx(f.read(f"{group}/Mat_{m}_Vfrac"), order, 1)
            if f.exists(f"{group}/Mat_{m}_S"):
                S = _to_zyx(f.read(f"{group}/Mat_{m}_S"), order, 1).astype(np.float32)
                vox[m - 1, ..., 0] = S
                th = _to_zyx(f.read(f"{group}/Mat_{m}_Theta"), order, 1).astype(np.float32)
                ps = _to_zyx(f.read(f"{group}/Mat_{m}_Psi"), order, 1).astype(np.float32)
                vox[m - 1, ..., 1] = np.where(S == 0, np.float32(0), th)
                vox[m - 1, ..., 2] = np.where(S == 0, np.float32(0), ps)
        else:
            al = f.read(f"{group}/Mat_{m}_alignment")
            if al.ndim != 4:
                raise ValueError(f"expected a 4D array for Mat_{m}_alignment, found {al.ndim}D")
            vox[m - 1, ..., 0:3] = _to_zyx(al, order, 3)
            vox[m - 1, ..., 3] = _to_zyx(f.read(f"{group}/Mat_{m}_unaligned"), order, 1)
    return Morphology(nmat, phys, order, (X, Y, Z), vox)


# ---------------------------------------------------------------------------
# writer
# ---------------------------------------------------------------------------
class _Writer:
    """Builds a file of the supported subset in memory: superblock 0,
    symbol-table groups, contiguous little-endian datasets, vlen-string
    DIMENSION_LABELS attributes (one global heap collection per file)."""

    def __init__(self):
        self.root = {}  # name -> dict (group) | (array, labels)

    def add(self, path: str, array: np.ndarray, labels=None):
        parts = [p for p in path.split("/") if p]
        g = self.root
        for p in parts[:-1]:
            g = g.setdefault(p, {})
        g[parts[-1]] = (np.ascontiguousarray(array), labels)

    # encoding helpers -----------------------------------------------------------------
    @staticmethod
    def _msg(mtype, body, flags=0):
        body = body + b"\0" * ((-len(body)) % 8)
        return struct.pack("<HHB3x", mtype, len(body), flags) + body

    @staticmethod
    def _dtype_msg(dt: np.dtype):
        dt = np.dtype(dt)
        if dt.kind == "f":
            if dt.itemsize == 4:
                props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            else:
                props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            # little endian, implied-msb mantissa normalisation, sign bit at the top
            return struct.pack("<BBBBI", 0x11, 0x20, 8 * dt.itemsize - 1, 0x00, dt.itemsize) + props
        if dt.kind in "iu":
            bits = 0x08 if dt.kind == "i" else 0
            return struct.pack("<BBBBI", 0x10, bits, 0, 0, dt.itemsize) + struct.pack("<HH", 0, 8 * dt.itemsize)
        raise ValueError(f"dtype {dt} cannot be written")

    @staticmethod
    def _space_msg(shape):
        body = struct.pack("<BBBB4x", 1, len(shape), 0, 0)
        return body + b"".join(struct.pack("<Q", int(n)) for n in shape)

    def _header(self, msgs):
        blob = b"".join(msgs)
        return struct.pack("<BBHII4x", 1, 0, len(msgs), 1, len(blob)) + blob

    GROUP_BTREE_K = 16  # group internal node K (superblock): B-tree nodes hold 2K children

    def tobytes(self) -> bytes:
        out = bytearray(b"\0" * 96)  # superblock (filled at the end)
        heap_objects = []  # global heap: strings

        def max_members(g):
            return max([len(g)] + [max_members(v) for v in g.values() if isinstance(v, dict)])

        # group leaf node K (superblock): every group's entries fit one symbol node of 2K entries
        leaf_k = max(4, (max_members(self.root) + 1) // 2)
        tree_k = self.GROUP_BTREE_K

        def alloc(data: bytes, align=8):
            pad = (-len(out)) % align
            out.extend(b"\0" * pad)
            addr = len(out)
            out.extend(data)
            return addr

        def write_dataset(arr, labels):
            arr = np.asarray(arr)
            le = arr.astype(arr.dtype.newbyteorder("<"))
            data_addr = alloc(le.tobytes(), 8) if arr.size else UNDEF
            msgs = [self._msg(0x01, self._space_msg(arr.shape)),
                    self._msg(0x03, self._dtype_msg(arr.dtype), flags=1),
                    self._msg(0x08, struct.pack("<BBQQ", 3, 1, data_addr, le.nbytes))]
            if labels:
                ids = []
                for lab in labels:
                    heap_objects.append(lab.encode())
                    ids.append(len(heap_objects))
                name = b"DIMENSION_LABELS\0"
                # vlen string of 1-byte fixed-point characters, as libhdf5 stores dimension labels
                dtype = struct.pack("<BBBBI", 0x19, 0x01, 0x00, 0x00, 16) + struct.pack("<BBBBIHH", 0x10, 0, 0, 0, 1, 0, 8)
                space = self._space_msg((len(labels),))
                vals = b"".join(struct.pack("<IQI", len(heap_objects[i - 1]), 0xC011C011C011C011, i) for i in ids)
                pad = lambda b: b + b"\0" * ((-len(b)) % 8)  # noqa: E731
                body = struct.pack("<BBHHH", 1, 0, len(name), len(dtype), len(space)) + pad(name) + pad(dtype) + \
                    pad(space) + vals
                msgs.append(self._msg(0x0C, body))
            return alloc(self._header(msgs))

        def write_group(members: dict):
            names = sorted(members)
            # local heap: "" at 0, then the names
            heap_data = bytearray(b"\0" * 8)
            offs = {}
            for n in names:
                offs[n] = len(heap_data)
                heap_data.extend(n.encode() + b"\0")
                heap_data.extend(b"\0" * ((-len(heap_data)) % 8))
            entries = []
            for n in names:
                v = members[n]
                if isinstance(v, dict):
                    hdr, scratch = write_group(v)
                    entries.append(struct.pack("<QQI4x", offs[n], hdr, 1) + struct.pack("<QQ", *scratch))
                else:
                    hdr = write_dataset(*v)
                    entries.append(struct.pack("<QQI4x", offs[n], hdr, 0) + b"\0" * 16)
            heap_data_addr = alloc(bytes(heap_data))
            heap_addr = alloc(b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), UNDEF, heap_data_addr))
            # one symbol node holding every entry (room for 2 leaf_k), one leaf B-tree node
            snod = b"SNOD" + struct.pack("<BBH", 1, 0, len(entries)) + b"".join(entries)
            snod += b"\0" * (40 * (2 * leaf_k - len(entries)))
            snod_addr = alloc(snod)
            last_key = offs[names[-1]] if names else 0
            tree = b"TREE" + struct.pack("<BBHQQ", 0, 0, 1 if entries else 0, UNDEF, UNDEF)
            tree += struct.pack("<QQQ", 0, snod_addr, last_key)
            tree += b"\0" * (8 * (2 * tree_k + 1) + 8 * (2 * tree_k) - 24)  # the node's full size
            tree_addr = alloc(tree)
            hdr = alloc(self._header([self._msg(0x11, struct.pack("<QQ", tree_addr, heap_addr))]))
            return hdr, (tree_addr, heap_addr)

        root_hdr, root_scratch = write_group(self.root)
        # global heap collection with every label string
        if heap_objects:
            objs = bytearray()
            for i, s in enumerate(heap_objects, 1):
                objs.extend(struct.pack("<HH4xQ", i, 1, len(s)) + s + b"\0" * ((-len(s)) % 8))
            size = max(4096, 16 + len(objs) + 16)
            coll = b"GCOL" + struct.pack("<B3xQ", 1, size) + bytes(objs)
            free = size - len(coll)
            coll += struct.pack("<HH4xQ", 0, 0, free) if free >= 16 else b""  # free space, its header included
            coll += b"\0" * (size - len(coll))
            gaddr = alloc(coll)
            out[:] = out.replace(struct.pack("<Q", 0xC011C011C011C011), struct.pack("<Q", gaddr))
        eof = len(out)
        sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", leaf_k, tree_k, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
        sb += struct.pack("<QQI4x", 0, root_hdr, 1) + struct.pack("<QQ", *root_scratch)
        out[0:len(sb)] = sb
        return bytes(out)


def write(path: str, datasets: dict):
    """Writes {"group/.../name": (array, labels or None)} to `path`."""
    w = _Writer()
    for k, v in datasets.items():
        arr, labels = v if isinstance(v, tuple) else (v, None)
        w.add(k, arr, labels)
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(path, "wb") as f:
        f.write(w.tobytes())


# ---------------------------------------------------------------------------
# CyRSoXS output files
# ---------------------------------------------------------------------------
def write_scattering(inp, data: np.ndarray, dir_name: str = "HDF5"):
    """One Energy_<E:.2f>.h5 per energy (include/utils.h:38-87)."""
    X, Y, _ = inp.voxelDims
    ks = np.asarray(inp.kVectors or [[0.0, 0.0, 1.0]], np.float32).reshape(-1, 3)
    nk, P = ks.shape[0], X * Y
    flat = np.asarray(data, np.float32).reshape(-1)
    for e, energy in enumerate(inp.energies):
        ds = {"KIDList/KVec": (ks, None)}
        for k in range(nk):
            off = (e * nk + k) * P
            ds[f"K{k}/projection"] = (flat[off:off + P].reshape(Y, X), ["Qy", "Qx"])
        write(os.path.join(dir_name, f"Energy_{float(np.float32(energy)):.2f}.h5"), ds)


def write_polarization(inp, p):
    """Polarization/Polarization{X,Y,Z}.h5 with p{X,Y,Z} [Z][Y][X][2] (writeH5.h:77-110)."""
    X, Y, Z = inp.voxelDims
    for name, arr in zip("XYZ", p):
        a = np.asarray(arr, np.complex64).reshape(Z, Y, X)
        re_im = np.stack([a.real, a.imag], axis=-1).astype(np.float32)
        write(os.path.join("Polarization", f"Polarization{name}.h5"), {f"p{name}": (re_im, ["Z", "Y", "X"])})


def write_morphology_dump(inp, voxels: np.ndarray, dir_name: str = "Morphology"):
    """Morphology/Morphology.h5 with Material_<m>/<component> [Z][Y][X] and the
    XDMF description Morphology/Morphology.xdmf that lets ParaView or VisIt
    open it (writeH5.h:117-243)."""
    X, Y, Z = inp.voxelDims
    names = ("S", "Theta", "Psi", "Vfrac") if inp.morphologyType == 0 else ("Sx", "Sy", "Sz", "UnalignedFraction")
    v = np.asarray(voxels, np.float32).reshape(inp.NUM_MATERIAL, Z, Y, X, 4)
    ds = {}
    for m in range(inp.NUM_MATERIAL):
        for c, n in enumerate(names):
            ds[f"Material_{m + 1}/{n}"] = (np.ascontiguousarray(v[m, ..., c]), ["Z", "Y", "X"])
    write(os.path.join(dir_name, "Morphology.h5"), ds)
    with open(os.path.join(dir_name, "Morphology.xdmf"), "w") as f:
        f.write(_xdmf(names, inp.NUM_MATERIAL, (Z, Y, X)))


def _xdmf(names, nmat, zyx):
    dims = " ".join(str(n) for n in zyx)
    attrs = []
    for c in names:
        for m in range(1, nmat + 1):
            attrs.append(f'    <Attribute Name="Mat_{m}_{c}" AttributeType="Scalar" Center="Cell">\n'
                         f'      <DataItem Dimensions="{dims}" NumberType="Float" Precision="4" Format="HDF">'
                         f"Morphology.h5:/Material_{m}/{c}</DataItem>\n    </Attribute>\n")
    return ('<?xml version="1.0" ?>\n<!DOCTYPE Xdmf SYSTEM "Xdmf.dtd" []>\n'
            '<Xdmf xmlns:xi="http://www.w3.org/2003/XInclude" Version="2.2">\n <Domain>\n'
            '  <Grid Name="morphology" GridType="Uniform">\n'
            f'    <Topology TopologyType="3DCORECTMesh" NumberOfElements="{dims}"/>\n'
            '    <Geometry GeometryType="ORIGIN_DXDYDZ">\n'
            '      <DataItem Name="origin" Dimensions="3" NumberType="Float" Precision="4" Format="XML">0.0 0.0 0.0</DataItem>\n'
            '      <DataItem Name="spacing" Dimensions="3" NumberType="Float" Precision="4" Format="XML">1.0 1.0 1.0</DataItem>\n'
            '    </Geometry>\n' + "".join(attrs) + '  </Grid>\n </Domain>\n</Xdmf>\n')
