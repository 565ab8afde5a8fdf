"""Minimal reader for netCDF-4 (HDF5) files as the reference writes them:
its restart files (mHM and mRM), flux/state outputs and input grids.

Written from the published HDF5 file-format specification, covering what
netCDF-C writes with HDF5's default (earliest) library bounds and newer
layouts: superblock version 0/1/2, version-1 and version-2 object headers
with continuation blocks, groups as symbol tables (version-1 B-tree of
symbol-table nodes plus a local heap) or as link messages / dense link
storage (fractal heap), dataspace / datatype (little-endian fixed and
floating point) / layout (version 3: contiguous, compact, chunked with a
version-1 B-tree index) / filter pipeline (deflate, shuffle, fletcher32)
messages.  Anything else raises NotImplementedError.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5File:
    def __init__(self, path: str):
        with open(path, "rb") as f:
            self.b = f.read()
        if self.b[:8] != SIG:
            raise ValueError("not an HDF5 file")
        ver = self.b[8]
        if ver in (2, 3):
            if self.b[9] != 8 or self.b[10] != 8:
                raise NotImplementedError("offset/length sizes other than 8")
            self.base = self.u64(12)
            self.root = self.u64(36)            # root group object header address
            return
        if ver not in (0, 1):
            raise NotImplementedError(f"superblock version {ver}")
        if self.b[13] != 8 or self.b[14] != 8:
            raise NotImplementedError("offset/length sizes other than 8")
        p = 24 + (4 if ver == 1 else 0)
        self.base = self.u64(p)
        root_entry = p + 32
        self.root = self.u64(root_entry + 8)   # object header address of the root group

    # ---- primitives ----
    def u8(self, p):
        return self.b[p]

    def u16(self, p):
        return struct.unpack_from("<H", self.b, p)[0]

    def u32(self, p):
        return struct.unpack_from("<I", self.b, p)[0]

    def u64(self, p):
        return struct.unpack_from("<Q", self.b, p)[0]

    def cstr(self, p):
        e = self.b.index(b"\0", p)
        return self.b[p:e].decode()

    # ---- object headers ----
    def messages(self, addr):
        """[(type, data bytes)] of an object header (version 1 or 2, with
        continuation blocks)."""
        if self.b[addr:addr + 4] == b"OHDR":
            return self._messages_v2(addr)
        if self.u8(addr) != 1:
            raise NotImplementedError(f"object header version {self.u8(addr)}")
        nmsg = self.u16(addr + 2)
        size = self.u32(addr + 8)
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            p, n = blocks.pop(0)
            end = p + n
            while p + 8 <= end and len(out) < nmsg:
                mtype, msize = self.u16(p), self.u16(p + 2)
                data = self.b[p + 8:p + 8 + msize]
                out.append((mtype, data))
                if mtype == 0x10:  # continuation
                    off, ln = struct.unpack_from("<QQ", data, 0)
                    blocks.append((off, ln))
                p += 8 + msize
        return out

    def _messages_v2(self, addr):
        if self.u8(addr + 4) != 2:
            raise NotImplementedError("object header v2 version")
        flags = self.u8(addr + 5)
        p = addr + 6
        if flags & 0x20:
            p += 16
        if flags & 0x10:
            p += 4
        w = 1 << (flags & 3)
        size = int.from_bytes(self.b[p:p + w], "little")
        p += w
        blocks = [(p, size)]
        out = []
        while blocks:
            q, n = blocks.pop(0)
            end = q + n - 4 if self.b[q - 4:q] == b"OCHK" else q + n
            while q + 4 <= end:
                mtype, msize = self.u8(q), self.u16(q + 1)
                q += 4 + (2 if flags & 0x04 else 0)
                data = self.b[q:q + msize]
                if mtype == 0x10:
                    off, ln = struct.unpack_from("<QQ", data, 0)
                    blocks.append((off + 4, ln - 4))  # skip the OCHK signature
                elif mtype != 0:
                    out.append((mtype, data))
                q += msize
        return out

    # ---- groups ----
    def group(self, addr=None) -> dict[str, int]:
        """name -> object header address of a group's members (symbol table,
        compact link messages or dense link storage in a fractal heap)."""
        addr = self.root if addr is None else addr
        msgs = self.messages(addr)
        out = {}
        for t, d in msgs:
            if t == 0x11:
                btree, heap = struct.unpack_from("<QQ", d, 0)
                return self._symbols(btree, heap)
            if t == 0x06:
                name, target = self._link(d, 0)[:2]
                out[name] = target
            if t == 0x02:
                flags = d[1]
                p = 2 + (8 if flags & 1 else 0)
                heap = struct.unpack_from("<Q", d, p)[0]
                if heap != UNDEF:
                    out.update(self._dense_links(heap))
        return out

    def _link(self, d, p):
        """Link message at d[p:]: (name, object address, length in bytes)."""
        p0 = p
        if d[p] != 1:
            raise ValueError("link message version")
        flags = d[p + 1]
        p += 2
        ltype = 0
        if flags & 0x08:
            ltype = d[p]
            p += 1
        if flags & 0x04:
            p += 8
        if flags & 0x10:
            p += 1
        w = 1 << (flags & 3)
        nlen = int.from_bytes(d[p:p + w], "little")
        p += w
        name = bytes(d[p:p + nlen]).decode()
        p += nlen
        if ltype != 0:
            raise NotImplementedError("soft or external links")
        target = struct.unpack_from("<Q", d, p)[0]
        return name, target, p + 8 - p0

    def _dense_links(self, heap):
        """Link messages stored as managed objects of a (write-once) fractal heap."""
        b = self.b
        if b[heap:heap + 4] != b"FRHP":
            raise ValueError("bad fractal heap")
        flags = b[heap + 8 + 1]
        q = heap + 4 + 1 + 2 + 2 + 1 + 4 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8
        width = self.u16(q)
        start = self.u64(q + 2)
        max_direct = self.u64(q + 10)
        max_heap_bits = self.u16(q + 18)
        root = self.u64(q + 22)
        rows = self.u16(q + 30)
        off_bytes = (max_heap_bits + 7) // 8
        cks = 4 if flags & 0x02 else 0
        out = {}

        def direct(addr, size):
            if b[addr:addr + 4] != b"FHDB":
                raise ValueError("bad direct block")
            p = addr + 5 + 8 + off_bytes + cks
            end = addr + size
            while p < end and b[p] == 1:
                name, target, n = self._link(b, p)
                out[name] = target
                p += n

        def indirect(addr, nrows):
            if b[addr:addr + 4] != b"FHIB":
                raise ValueError("bad indirect block")
            p = addr + 5 + 8 + off_bytes
            for r in range(nrows):
                size = start * (1 << max(0, r - 1))
                for _ in range(width):
                    child = self.u64(p)
                    p += 8
                    if child == UNDEF:
                        continue
                    if size <= max_direct:
                        direct(child, size)
                    else:
                        raise NotImplementedError("nested indirect blocks")

        if rows == 0:
            direct(root, start)
        else:
            indirect(root, rows)
        return out

    def _heap_data(self, heap):
        if self.b[heap:heap + 4] != b"HEAP":
            raise ValueError("bad local heap")
        return self.u64(heap + 24)

    def _symbols(self, btree, heap):
        hd = self._heap_data(heap)
        out = {}

        def walk(node):
            if self.b[node:node + 4] != b"TREE":
                raise ValueError("bad B-tree node")
            level, used = self.u8(node + 5), self.u16(node + 6)
            p = node + 24 + 8  # first key
            for _ in range(used):
                child = self.u64(p)
                if level > 0:
                    walk(child)
                else:
                    snod(child)
                p += 16
        def snod(addr):
            if self.b[addr:addr + 4] != b"SNOD":
                raise ValueError("bad symbol-table node")
            n = self.u16(addr + 6)
            for i in range(n):
                e = addr + 8 + 40 * i
                name = self.cstr(hd + self.u64(e))
                out[name] = self.u64(e + 8)
        walk(btree)
        return out

    # ---- datasets ----
    def read(self, name: str, group_addr=None) -> np.ndarray:
        addr = self.group(group_addr)[name]
        dims, dtype, layout, filters = None, None, None, []
        for t, d in self.messages(addr):
            if t == 0x01:
                dims = self._dataspace(d)
            elif t == 0x03:
                dtype = self._datatype(d)
            elif t == 0x08:
                layout = d
            elif t == 0x0B:
                filters = self._filters(d)
        if dims is None or dtype is None or layout is None:
            raise ValueError(f"{name}: not a dataset")
        return self._data(layout, dims, dtype, filters)

    def _dataspace(self, d):
        ver, ndim = d[0], d[1]
        p = 8 if ver == 1 else 4
        return tuple(struct.unpack_from("<Q", d, p + 8 * i)[0] for i in range(ndim))

    def _datatype(self, d):
        cls, size = d[0] & 0x0F, struct.unpack_from("<I", d, 4)[0]
        be = d[1] & 1
        if be:
            raise NotImplementedError("big-endian data")
        if cls == 1:
            return np.dtype({4: "<f4", 8: "<f8"}[size])
        if cls == 0:
            signed = (d[1] >> 3) & 1
            return np.dtype(("<i" if signed else "<u") + str(size))
        raise NotImplementedError(f"datatype class {cls}")

    def _filters(self, d):
        ver, n = d[0], d[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = struct.unpack_from("<H", d, p)[0]
            if ver == 1 or fid >= 256:
                nlen, _flags, nval = struct.unpack_from("<HHH", d, p + 2)
                p += 8
                p += (nlen + 7) // 8 * 8 if ver == 1 else nlen
            else:
                _flags, nval = struct.unpack_from("<HH", d, p + 2)
                p += 6
            vals = struct.unpack_from("<" + "I" * nval, d, p) if nval else ()
            p += 4 * nval
            if ver == 1 and nval % 2:
                p += 4
            out.append((fid, vals))
        return out

    def _data(self, lay, dims, dtype, filters):
        if lay[0] != 3:
            raise NotImplementedError(f"layout version {lay[0]}")
        cls = lay[1]
        count = int(np.prod(dims)) if dims else 1
        if cls == 0:  # compact
            n = struct.unpack_from("<H", lay, 2)[0]
            return np.frombuffer(lay[4:4 + n], dtype).reshape(dims).copy()
        if cls == 1:  # contiguous
            addr, size = struct.unpack_from("<QQ", lay, 2)
            if addr == UNDEF:
                return np.zeros(dims, dtype)
            return np.frombuffer(self.b, dtype, count, addr).reshape(dims).copy()
        if cls != 2:
            raise NotImplementedError(f"layout class {cls}")
        nd = lay[2]
        btree = struct.unpack_from("<Q", lay, 3)[0]
        cdims = struct.unpack_from("<" + "I" * nd, lay, 11)[:-1]   # last entry = element size
        out = np.zeros(dims, dtype)
        if btree == UNDEF:
            return out

        def walk(node):
            if self.b[node:node + 4] != b"TREE" or self.b[node + 4] != 1:
                raise ValueError("bad chunk B-tree node")
            level, used = self.u8(node + 5), self.u16(node + 6)
            ksize = 8 + 8 * nd
            p = node + 24
            for _ in range(used):
                csize, fmask = self.u32(p), self.u32(p + 4)
                offs = struct.unpack_from("<" + "Q" * (nd - 1), self.b, p + 8)
                child = self.u64(p + ksize)
                if level > 0:
                    walk(child)
                else:
                    raw = self.b[child:child + csize]
                    for i, (fid, vals) in reversed(list(enumerate(filters))):
                        if fmask & (1 << i):
                            continue
                        if fid == 1:
                            raw = zlib.decompress(raw)
                        elif fid == 2:
                            es = dtype.itemsize
                            a = np.frombuffer(raw, np.uint8).reshape(es, -1)
                            raw = a.T.tobytes()
                        elif fid == 3:
                            raw = raw[:-4]
                        else:
                            raise NotImplementedError(f"filter {fid}")
                    chunk = np.frombuffer(raw, dtype, int(np.prod(cdims))).reshape(cdims)
                    sl = tuple(slice(o, min(o + c, n)) for o, c, n in zip(offs, cdims, dims))
                    out[sl] = chunk[tuple(slice(0, s.stop - s.start) for s in sl)]
                p += ksize + 8
        walk(btree)
        return out
