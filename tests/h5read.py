"""A small reader of the HDF5 file format, written from the published format specification,
for the tests: it reads the files the library writes (outfile.thermal_conductivity_grid.hdf5)
and the reference's own HDF5 fixtures (written by libhdf5: superblock 0, version-1 object
headers, symbol-table groups, contiguous or chunked datasets with the deflate filter).

Supported: superblock 0/1 (and 2/3 with a root object header), object headers 1 and 2,
groups by symbol table (v1 B-tree + local heap) and by link messages, datasets of IEEE
floats, integers and fixed-length strings with contiguous, compact or chunked (v1 B-tree
index, deflate and shuffle filters) layout, and attributes of those types.

    f = H5File(path); f.datasets -> {name: ndarray}; f.attrs -> {name: value};
    f.dataset_attrs -> {name: {attr: value}}
"""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


class H5File:
    def __init__(self, path):
        self.buf = Path(path).read_bytes()
        b = self.buf
        if b[:8] != b"\x89HDF\r\n\x1a\n":
            raise ValueError("not an HDF5 file")
        ver = b[8]
        self.superblock_version = ver
        if ver in (0, 1):
            self.so, self.sl = b[13], b[14]
            self.leaf_k, self.internal_k = struct.unpack_from("<HH", b, 16)
            p = 24 + (4 if ver == 1 else 0)
            self.base, _, self.eof, _ = struct.unpack_from("<4Q", b, p)
            p += 32
            root_header = struct.unpack_from("<Q", b, p + 8)[0]
        else:
            self.so, self.sl = b[9], b[10]
            self.base, _, self.eof, root_header = struct.unpack_from("<4Q", b, 12)
        self.attrs, self.datasets, self.dataset_attrs, self.objects = {}, {}, {}, {}
        self.root = root_header
        msgs = self._messages(root_header)
        self.attrs = self._attributes(msgs)
        self._walk_group(msgs, "")

    # ------------------------------------------------------------------ object headers
    def _messages(self, addr):
        b = self.buf
        out = []
        if b[addr:addr + 4] == b"OHDR":
            flags = b[addr + 5]
            p = addr + 6
            if flags & 0x20:
                p += 16
            if flags & 0x10:
                p += 4
            nsz = 1 << (flags & 3)
            size = int.from_bytes(b[p:p + nsz], "little")
            p += nsz
            self._v2_chunk(p, p + size, flags, out)
            return out
        version, _, nmsg, _, hsize = struct.unpack_from("<BBHII", b, addr)
        if version != 1:
            raise ValueError(f"object header version {version}")
        self._v1_chunk(addr + 16, addr + 16 + hsize, out)
        return out

    def _v1_chunk(self, p, end, out):
        b = self.buf
        while p + 8 <= end:
            mtype, msize, mflags = struct.unpack_from("<HHB", b, p)
            data = b[p + 8:p + 8 + msize]
            if mtype == 0x10:  # continuation
                a, ln = struct.unpack_from("<QQ", data)
                self._v1_chunk(a, a + ln, out)
            elif mtype != 0:
                out.append((mtype, data))
            p += 8 + msize

    def _v2_chunk(self, p, end, flags, out):
        b = self.buf
        while p + 4 <= end - 4:
            mtype, msize, mflags = struct.unpack_from("<BHB", b, p)
            p += 4
            if flags & 0x04:
                p += 2
            data = b[p:p + msize]
            if mtype == 0x10:
                a, ln = struct.unpack_from("<QQ", data)
                self._v2_chunk(a + 4, a + ln - 4, flags, out)
            elif mtype != 0:
                out.append((mtype, data))
            p += msize

    # ------------------------------------------------------------------ groups
    def _heap_string(self, heap_addr, off):
        b = self.buf
        assert b[heap_addr:heap_addr + 4] == b"HEAP"
        data_addr = struct.unpack_from("<Q", b, heap_addr + 24)[0]
        s = data_addr + off
        return b[s:b.index(b"\0", s)].decode()

    def _walk_group(self, msgs, prefix):
        for mtype, data in msgs:
            if mtype == 0x11:  # symbol table
                btree, heap = struct.unpack_from("<QQ", data)
                for name, addr in self._btree_group(btree, heap):
                    self._object(prefix + name, addr)
            elif mtype == 0x06:  # link message (compact storage of a new-style group)
                name, addr = self._link(data)
                if addr is not None:
                    self._object(prefix + name, addr)

    def _link(self, d):
        version, flags = d[0], d[1]
        p = 2
        ltype = 0
        if flags & 0x08:
            ltype = d[p]
            p += 1
        if flags & 0x04:
            p += 8
        if flags & 0x10:
            p += 1
        nsz = 1 << (flags & 3)
        ln = int.from_bytes(d[p:p + nsz], "little")
        p += nsz
        name = d[p:p + ln].decode()
        p += ln
        if ltype != 0:
            return name, None
        return name, struct.unpack_from("<Q", d, p)[0]

    def _btree_group(self, addr, heap):
        b = self.buf
        assert b[addr:addr + 4] == b"TREE", "group B-tree signature"
        ntype, level, used = b[addr + 4], b[addr + 5], struct.unpack_from("<H", b, addr + 6)[0]
        p = addr + 8 + 16
        out = []
        for i in range(used):
            child = struct.unpack_from("<Q", b, p + 8)[0]
            p += 16
            if level > 0:
                out += self._btree_group(child, heap)
            else:
                assert b[child:child + 4] == b"SNOD"
                nsym = struct.unpack_from("<H", b, child + 6)[0]
                for k in range(nsym):
                    e = child + 8 + 40 * k
                    name_off, ohdr = struct.unpack_from("<QQ", b, e)
                    out.append((self._heap_string(heap, name_off), ohdr))
        return out

    def _object(self, name, addr):
        msgs = self._messages(addr)
        types = {t for t, _ in msgs}
        self.objects[name] = addr
        if 0x11 in types or 0x06 in types or 0x02 in types:
            self._walk_group(msgs, name + "/")
            return
        if 0x08 in types:
            self.datasets[name] = self._dataset(msgs)
            self.dataset_attrs[name] = self._attributes(msgs)

    # ------------------------------------------------------------------ datatypes, dataspaces
    @staticmethod
    def _dataspace(d):
        version, rank, flags = d[0], d[1], d[2]
        p = 8 if version == 1 else 4
        if version == 2 and d[3] == 0:
            return ()  # scalar
        dims = struct.unpack_from(f"<{rank}Q", d, p)
        return tuple(int(x) for x in dims)

    @staticmethod
    def _datatype(d):
        cls, bits, size = d[0] & 0x0F, d[1:4], struct.unpack_from("<I", d, 4)[0]
        if cls == 1:
            if bits[0] & 1:
                raise ValueError("big-endian float")
            return np.dtype(f"<f{size}")
        if cls == 0:
            signed = bool(bits[0] & 0x08)
            return np.dtype(f"<{'i' if signed else 'u'}{size}")
        if cls == 3:
            return np.dtype(f"S{size}")
        raise ValueError(f"datatype class {cls}")

    def _attributes(self, msgs):
        out = {}
        for mtype, d in msgs:
            if mtype != 0x0C:
                continue
            version = d[0]
            nlen, tlen, slen = struct.unpack_from("<HHH", d, 2)
            if version == 1:
                p = 8
                pad = lambda x: (x + 7) // 8 * 8
                name = d[p:p + nlen].split(b"\0")[0].decode()
                p += pad(nlen)
                dt = self._datatype(d[p:p + tlen])
                p += pad(tlen)
                shape = self._dataspace(d[p:p + slen])
                p += pad(slen)
            else:
                p = 8 if version == 2 else 9
                name = d[p:p + nlen].split(b"\0")[0].decode()
                p += nlen
                dt = self._datatype(d[p:p + tlen])
                p += tlen
                shape = self._dataspace(d[p:p + slen])
                p += slen
            cnt = int(np.prod(shape)) if shape else 1
            arr = np.frombuffer(d[p:p + cnt * dt.itemsize], dt)
            if dt.kind == "S":
                v = arr[0].split(b"\0")[0].decode()
            else:
                v = arr.reshape(shape) if shape else arr[0]
            out[name] = v
        return out

    # ------------------------------------------------------------------ datasets
    def _dataset(self, msgs):
        dt = shape = layout = None
        filters = []
        for mtype, d in msgs:
            if mtype == 0x01:
                shape = self._dataspace(d)
            elif mtype == 0x03:
                dt = self._datatype(d)
            elif mtype == 0x08:
                layout = d
            elif mtype == 0x0B:
                filters = self._filters(d)
        count = int(np.prod(shape)) if shape else 1
        version, cls = layout[0], layout[1]
        if version != 3:
            raise ValueError(f"layout message version {version}")
        if cls == 0:  # compact
            size = struct.unpack_from("<H", layout, 2)[0]
            raw = layout[4:4 + size]
        elif cls == 1:  # contiguous
            addr, size = struct.unpack_from("<QQ", layout, 2)
            raw = self.buf[addr:addr + size] if addr != UNDEF else bytes(count * dt.itemsize)
        elif cls == 2:  # chunked, v1 B-tree index
            rank = layout[2]
            addr = struct.unpack_from("<Q", layout, 3)[0]
            cdims = struct.unpack_from(f"<{rank}I", layout, 11)
            return self._chunked(addr, shape, cdims[:-1], dt, filters)
        else:
            raise ValueError(f"layout class {cls}")
        arr = np.frombuffer(raw[:count * dt.itemsize], dt)
        return arr.reshape(shape) if shape else arr[0]

    @staticmethod
    def _filters(d):
        version, n = d[0], d[1]
        p = 8 if version == 1 else 2
        out = []
        for _ in range(n):
            fid = struct.unpack_from("<H", d, p)[0]
            if version == 1 or fid >= 256:
                nlen = struct.unpack_from("<H", d, p + 2)[0]
                ncv = struct.unpack_from("<H", d, p + 6)[0]
                p += 8 + ((nlen + 7) // 8 * 8 if version == 1 else nlen)
            else:
                ncv = struct.unpack_from("<H", d, p + 4)[0]
                p += 6
            p += 4 * ncv
            if version == 1 and ncv % 2:
                p += 4
            out.append(fid)
        return out

    def _chunked(self, addr, shape, cdims, dt, filters):
        out = np.zeros(shape, dt)
        rank = len(shape)
        for offs, raw, mask in self._btree_chunks(addr, rank):
            for i, fid in enumerate(reversed(filters)):
                if mask & (1 << (len(filters) - 1 - i)):
                    continue
                if fid == 1:
                    raw = zlib.decompress(raw)
                elif fid == 2:
                    n = len(raw) // dt.itemsize
                    raw = np.frombuffer(raw, np.uint8).reshape(dt.itemsize, n).T.tobytes()
                else:
                    raise ValueError(f"filter {fid}")
            chunk = np.frombuffer(raw, dt)[: int(np.prod(cdims))].reshape(cdims)
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
            out[sl] = chunk[tuple(slice(0, x.stop - x.start) for x in sl)]
        return out

    def _btree_chunks(self, addr, rank):
        b = self.buf
        assert b[addr:addr + 4] == b"TREE", "chunk B-tree signature"
        level, used = b[addr + 5], struct.unpack_from("<H", b, addr + 6)[0]
        ksz = 8 + 8 * (rank + 1)
        p = addr + 24
        for i in range(used):
            size, mask = struct.unpack_from("<II", b, p)
            offs = struct.unpack_from(f"<{rank}Q", b, p + 8)
            child = struct.unpack_from("<Q", b, p + ksz)[0]
            p += ksz + 8
            if level > 0:
                yield from self._btree_chunks(child, rank)
            else:
                yield offs, b[child:child + size], mask
