"""Puffin's HDF5 dump files on the host: read the reference's particle and
field dumps (to start a GPU run from them or to compare against them) and
write dumps in the same layout (to hand a GPU run back to the reference).

Layout (puffin/lib/io/hdf5_puff.f90, h5_in.f90:130-330, 735-1000):
* particle file: dataset ``electrons`` of shape (n, 7) holding x, y, z2, px,
  py (the stored -py), gamma, chi for each macroparticle, with the resume
  attributes (iCsteps, istep, iUnd_cr, ..., zbarLocal, zbarTotal, ...);
* field file: dataset ``aperp`` of shape (2, nz2, ny, nx) (3D) or (2, nz2)
  (1D), real then imaginary part, with the same attributes.

No HDF5 library exists on these machines, so both directions are written
here against the file-format specification: the reader handles superblock
versions 0 and 1, version-1 object headers, version-1 group B-trees, local
heaps, contiguous and compact layouts and version-1 attributes (what the
reference's files use); the writer emits that same classic subset (superblock
0, one root group, contiguous IEEE little-endian datasets, scalar and 1-D
attributes).  The reference's VizSchema metadata groups are not written.
"""
from __future__ import annotations

import struct

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"


class H5Reader:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.buf = f.read()
        if self.buf[:8] != SIG:
            raise ValueError(f"{path}: not an HDF5 file")
        b = self.buf
        ver = b[8]
        if ver not in (0, 1):
            raise ValueError(f"unsupported superblock version {ver}")
        self.so = b[13]
        self.sl = b[14]
        p = 16 + 4 + 4
        if ver == 1:
            p += 4
        self.base = self._off(p)
        p += 4 * self.so
        # root group symbol table entry
        self.root_hdr = self._off(p + self.so)
        cache_type = struct.unpack_from("<I", b, p + 2 * self.so)[0]
        self.root_scratch = p + 2 * self.so + 8
        self.root_cache_type = cache_type

    # -- primitive readers -------------------------------------------------
    def _off(self, p):
        return int.from_bytes(self.buf[p:p + self.so], "little")

    def _len(self, p):
        return int.from_bytes(self.buf[p:p + self.sl], "little")

    # -- object headers ----------------------------------------------------
    def messages(self, addr):
        b = self.buf
        if b[addr] != 1:
            raise ValueError(f"object header version {b[addr]} unsupported")
        nmsg = struct.unpack_from("<H", b, addr + 2)[0]
        hsize = struct.unpack_from("<I", b, addr + 8)[0]
        blocks = [(addr + 16, hsize)]
        out = []
        while blocks and len(out) < nmsg:
            start, size = blocks.pop(0)
            p = start
            while p < start + size and len(out) < nmsg:
                mtype, msize, mflags = struct.unpack_from("<HHB", b, p)
                data = p + 8
                if mtype == 0x10:  # continuation
                    blocks.append((self._off(data), self._len(data + self.so)))
                out.append((mtype, data, msize))
                p = data + msize
        return out

    # -- groups ------------------------------------------------------------
    def _heap_data(self, heap_addr):
        if self.buf[heap_addr:heap_addr + 4] != b"HEAP":
            raise ValueError("bad local heap")
        return self._off(heap_addr + 8 + 2 * self.sl)

    def _name(self, heap_data, off):
        end = self.buf.index(b"\0", heap_data + off)
        return self.buf[heap_data + off:end].decode()

    def _walk_btree(self, node, heap_data, out):
        b = self.buf
        if b[node:node + 4] != b"TREE":
            raise ValueError("bad group B-tree node")
        level = b[node + 5]
        used = struct.unpack_from("<H", b, node + 6)[0]
        p = node + 8 + 2 * self.so
        p += self.sl  # key 0
        for _ in range(used):
            child = self._off(p)
            p += self.so + self.sl
            if level > 0:
                self._walk_btree(child, heap_data, out)
            else:
                self._read_snod(child, heap_data, out)

    def _read_snod(self, addr, heap_data, out):
        b = self.buf
        if b[addr:addr + 4] != b"SNOD":
            raise ValueError("bad symbol table node")
        n = struct.unpack_from("<H", b, addr + 6)[0]
        p = addr + 8
        esz = 2 * self.so + 8 + 16
        for _ in range(n):
            name = self._name(heap_data, self._off(p))
            out[name] = self._off(p + self.so)
            p += esz

    def group_members(self, hdr_addr):
        for mtype, data, _ in self.messages(hdr_addr):
            if mtype == 0x11:
                btree = self._off(data)
                heap = self._off(data + self.so)
                out = {}
                self._walk_btree(btree, self._heap_data(heap), out)
                return out
        return {}

    # -- datatypes / dataspaces ---------------------------------------------
    def _dtype(self, p):
        b = self.buf
        cls = b[p] & 0x0F
        bits = b[p + 1]
        size = struct.unpack_from("<I", b, p + 4)[0]
        order = ">" if bits & 1 else "<"
        if cls == 1:
            return np.dtype(f"{order}f{size}")
        if cls == 0:
            signed = bool(bits & 0x08)
            return np.dtype(f"{order}{'i' if signed else 'u'}{size}")
        if cls == 3:
            return np.dtype(f"S{size}")
        raise ValueError(f"datatype class {cls} unsupported")

    def _dspace(self, p):
        b = self.buf
        ver = b[p]
        ndim = b[p + 1]
        if ver == 1:
            q = p + 8
        elif ver == 2:
            if b[p + 3] == 0:  # scalar
                return ()
            q = p + 4
        else:
            raise ValueError(f"dataspace version {ver}")
        return tuple(self._len(q + i * self.sl) for i in range(ndim))

    # -- attributes ----------------------------------------------------------
    def attributes(self, hdr_addr):
        out = {}
        for mtype, data, _ in self.messages(hdr_addr):
            if mtype != 0x0C:
                continue
            b = self.buf
            ver = b[data]
            if ver != 1:
                continue
            nsz, tsz, ssz = struct.unpack_from("<HHH", b, data + 2)
            p = data + 8
            name = b[p:p + nsz].split(b"\0")[0].decode()
            p += (nsz + 7) // 8 * 8
            dt = self._dtype(p)
            p += (tsz + 7) // 8 * 8
            shape = self._dspace(p)
            p += (ssz + 7) // 8 * 8
            count = int(np.prod(shape)) if shape else 1
            arr = np.frombuffer(b, dtype=dt, count=count, offset=p)
            val = arr.reshape(shape) if shape else arr[0]
            if dt.kind == "S":
                val = val.tobytes().split(b"\0")[0].decode() if not shape else val
            out[name] = val
        return out

    # -- datasets -------------------------------------------------------------
    def dataset(self, hdr_addr):
        dt = shape = None
        layout = None
        for mtype, data, msize in self.messages(hdr_addr):
            if mtype == 0x01:
                shape = self._dspace(data)
            elif mtype == 0x03:
                dt = self._dtype(data)
            elif mtype == 0x08:
                layout = (data, msize)
        if dt is None or shape is None or layout is None:
            raise ValueError("object is not a dataset")
        data, _ = layout
        ver = self.buf[data]
        count = int(np.prod(shape)) if shape else 1
        if ver == 3:
            cls = self.buf[data + 1]
            if cls == 1:
                addr = self._off(data + 2)
            elif cls == 0:
                addr = data + 4
            else:
                raise ValueError("chunked layout unsupported")
        elif ver in (1, 2):
            ndim = self.buf[data + 1]
            cls = self.buf[data + 2]
            if cls != 1:
                raise ValueError("only contiguous v1/v2 layouts supported")
            addr = self._off(data + 8)
            del ndim
        else:
            raise ValueError(f"layout version {ver}")
        arr = np.frombuffer(self.buf, dtype=dt, count=count, offset=addr)
        return arr.reshape(shape).astype(dt.newbyteorder("="))

    # -- convenience ----------------------------------------------------------
    def root(self):
        return self.root_hdr

    def tree(self, addr=None, prefix=""):
        """Yield (path, header address, kind) for every object below addr."""
        addr = self.root_hdr if addr is None else addr
        for name, child in sorted(self.group_members(addr).items()):
            kinds = {m for m, _, _ in self.messages(child)}
            kind = "group" if 0x11 in kinds else "dataset"
            path = f"{prefix}/{name}"
            yield path, child, kind
            if kind == "group":
                yield from self.tree(child, path)


# ---------------------------------------------------------------------------
# writer
# ---------------------------------------------------------------------------
UNDEF = 0xFFFFFFFFFFFFFFFF


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * ((-len(b)) % 8)


def _dtype_msg(dt: np.dtype) -> bytes:
    dt = np.dtype(dt)
    if dt.kind == "f":
        size = dt.itemsize
        if size == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
        else:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
        sign = 8 * size - 1
        return bytes([0x11, 0x20, sign, 0x00]) + struct.pack("<I", size) + props
    if dt.kind in "iu":
        size = dt.itemsize
        bits = 0x08 if dt.kind == "i" else 0x00
        return bytes([0x10, bits, 0, 0]) + struct.pack("<I", size) + struct.pack("<HH", 0, 8 * size)
    raise ValueError(f"dtype {dt} not supported by the writer")


def _dspace_msg(shape) -> bytes:
    out = bytes([1, len(shape), 0, 0]) + b"\0" * 4
    for n in shape:
        out += struct.pack("<Q", n)
    return out


def _message(mtype: int, body: bytes, flags: int = 0) -> bytes:
    body = _pad8(body)
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _attribute(name: str, value) -> bytes:
    arr = np.asarray(value)
    if arr.dtype.kind in "iu":
        arr = arr.astype("<i8")
    elif arr.dtype.kind == "f":
        arr = arr.astype("<f8")
    elif arr.dtype.kind == "b":
        arr = arr.astype("<i8")
    else:
        raise ValueError(f"attribute {name}: numeric values only")
    nm = name.encode() + b"\0"
    dt = _dtype_msg(arr.dtype)
    ds = _dspace_msg(arr.shape)
    head = struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(ds))
    return _message(0x0C, head + _pad8(nm) + _pad8(dt) + _pad8(ds) + arr.tobytes())


def write(path, datasets):
    """Write an HDF5 file holding the given datasets in its root group.
    ``datasets``: {name: (array, {attribute name: number or 1-D array})}."""
    names = sorted(datasets)
    if len(names) > 8:
        raise ValueError("at most 8 datasets per file (one symbol table node)")
    out = bytearray()

    def alloc(nbytes):
        off = len(out)
        out.extend(b"\0" * nbytes)
        return off

    # superblock (v0): 8 sig + 16 fixed + 4*8 addresses + root entry (40)
    sb = alloc(8 + 16 + 32 + 40)
    # local heap with the names (offset 0: the empty name)
    heap_data = b"\0" * 8
    name_off = {}
    for n in names:
        name_off[n] = len(heap_data)
        heap_data += _pad8(n.encode() + b"\0")
    heap = alloc(32)
    heap_seg = alloc(len(heap_data))
    out[heap_seg:heap_seg + len(heap_data)] = heap_data
    out[heap:heap + 32] = b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack(
        "<QQQ", len(heap_data), UNDEF, heap_seg)
    # symbol table node (2K = 8 entries) and group B-tree
    snod = alloc(8 + 8 * 40)
    btree = alloc(8 + 16 + 3 * 8)
    # datasets: object headers then data
    hdrs = {}
    for n in names:
        arr, attrs = datasets[n]
        arr = np.ascontiguousarray(arr)
        if arr.dtype.kind == "f":
            arr = arr.astype("<f8")
        msgs = _message(0x01, _dspace_msg(arr.shape))
        msgs += _message(0x03, _dtype_msg(arr.dtype), flags=1)
        msgs += _message(0x05, bytes([2, 2, 2, 0]))  # fill value v2: early, never written, undefined
        layout_at = len(msgs) + 8  # offset of the layout body in the message block
        msgs += _message(0x08, bytes([3, 1]) + struct.pack("<QQ", 0, arr.nbytes))
        for k in sorted(attrs):
            msgs += _attribute(k, attrs[k])
        hdr = alloc(16 + len(msgs))
        nmsg = 4 + len(attrs)
        out[hdr:hdr + 16] = struct.pack("<BBHII4x", 1, 0, nmsg, 1, len(msgs))
        out[hdr + 16:hdr + 16 + len(msgs)] = msgs
        data = alloc(arr.nbytes + ((-arr.nbytes) % 8))
        out[data:data + arr.nbytes] = arr.tobytes()
        struct.pack_into("<Q", out, hdr + 16 + layout_at + 2, data)
        hdrs[n] = hdr
    # root group object header: the symbol table message
    rmsg = _message(0x11, struct.pack("<QQ", btree, heap))
    root = alloc(16 + len(rmsg))
    out[root:root + 16] = struct.pack("<BBHII4x", 1, 0, 1, 1, len(rmsg))
    out[root + 16:root + 16 + len(rmsg)] = rmsg
    # symbol table node entries (sorted by name)
    ent = b""
    for n in names:
        ent += struct.pack("<QQII16x", name_off[n], hdrs[n], 0, 0)
    out[snod:snod + 8] = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(names))
    out[snod + 8:snod + 8 + len(ent)] = ent
    # B-tree (type 0 = group, level 0, one child): key0, child, key1
    last = name_off[names[-1]] if names else 0
    out[btree:btree + 24] = b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", 1 if names else 0,
                                                                 UNDEF, UNDEF)
    out[btree + 24:btree + 48] = struct.pack("<QQQ", 0, snod, last)
    # superblock
    out[sb:sb + 8] = b"\x89HDF\r\n\x1a\n"
    out[sb + 8:sb + 24] = bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0)
    out[sb + 24:sb + 56] = struct.pack("<QQQQ", 0, UNDEF, len(out), UNDEF)
    out[sb + 56:sb + 96] = struct.pack("<QQII", 0, root, 1, 0) + struct.pack("<QQ", btree, heap)
    with open(path, "wb") as f:
        f.write(bytes(out))


# ---------------------------------------------------------------------------
# Puffin dumps
# ---------------------------------------------------------------------------
PARTICLE_COLUMNS = ("x", "y", "z2", "px", "py", "gam", "chi")
RESUME_KEYS = ("iCsteps", "istep", "iUnd_cr", "iChic_cr", "iDrift_cr", "iQuad_cr",
               "iModulation_cr", "iL", "iWrite_cr", "zbarLocal", "zbarTotal", "zbarInter",
               "zLocal", "zTotal", "zInter", "time")


def _find(reader, name):
    members = reader.group_members(reader.root_hdr)
    if name not in members:
        raise KeyError(f"no dataset {name!r} in the file")
    return members[name]


def read_particles(path):
    """(beam dict x, y, z2, px, py, gam, chi; attributes) of a particle dump."""
    r = H5Reader(path)
    addr = _find(r, "electrons")
    e = r.dataset(addr)
    if e.ndim != 2 or e.shape[1] != 7:
        raise ValueError(f"electrons dataset of shape {e.shape}, expected (n, 7)")
    beam = {k: np.ascontiguousarray(e[:, j], dtype=np.float64) for j, k in enumerate(PARTICLE_COLUMNS)}
    return beam, r.attributes(addr)


def read_field(path):
    """(re, im flattened x fastest over the outer mesh; shape of the dataset;
    attributes) of a field dump."""
    r = H5Reader(path)
    addr = _find(r, "aperp")
    a = r.dataset(addr)
    if a.shape[0] != 2:
        raise ValueError(f"aperp dataset of shape {a.shape}, expected (2, ...)")
    return (np.ascontiguousarray(a[0].ravel(), dtype=np.float64),
            np.ascontiguousarray(a[1].ravel(), dtype=np.float64), a.shape, r.attributes(addr))


def write_particles(path, beam, attrs=None):
    e = np.stack([np.asarray(beam[k], dtype=np.float64) for k in PARTICLE_COLUMNS], axis=1)
    write(path, {"electrons": (e, dict(attrs or {}))})


def write_field(path, re, im, mesh, attrs=None):
    """mesh = (nx, ny, nz2); a 1D mesh (1, 1, nz2) is written as (2, nz2)."""
    nx, ny, nz2 = mesh
    shape = (2, nz2) if nx * ny == 1 else (2, nz2, ny, nx)
    a = np.stack([np.asarray(re, dtype=np.float64), np.asarray(im, dtype=np.float64)])
    write(path, {"aperp": (a.reshape(shape), dict(attrs or {}))})
