"""Minimal read-only HDF5 reader for the reference's golden dump files.

Test infrastructure only: it exists so that ``make_golden.py`` can turn the
reference's expected HDF5 outputs (``test/expected/f1main_expected_*.h5``) into
small committed fixtures without h5py, which is not installed here.

Supported subset (what those files use): superblock version 0/1, version-1
object headers with continuation blocks, version-1 group B-trees with symbol
table nodes and local heaps, contiguous and compact layouts, fixed-point,
floating-point and fixed-length string datatypes, and version-1 attributes.
"""
from __future__ import annotations

import struct

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"


class H5File:
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
