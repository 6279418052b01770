"""Minimal read-only HDF5 reader (fixture generation only; no libhdf5/h5py here).

Covers what DAMASK's DADF5 result files of the reference's test resources use:
superblock v0/v1, version-1 object headers with continuation blocks, old-style
groups (symbol-table message, v1 group B-tree, SNOD nodes, local heap), dataspace
v1/v2, fixed-point and IEEE float datatypes, contiguous/compact/chunked layouts (v1
chunk B-tree) and the deflate, shuffle and fletcher32 filters.  Format facts follow
the public "HDF5 File Format Specification Version 2.0".
"""
import struct
import zlib

import numpy as np


class HDF5File:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        b = self.b
        if b[:8] != b"\x89HDF\r\n\x1a\n":
            raise ValueError("not an HDF5 file")
        ver = b[8]
        if ver not in (0, 1):
            raise NotImplementedError(f"superblock v{ver}")
        self.so, self.sl = b[13], b[14]
        p = 24 if ver == 0 else 28
        self.base, _fs, _eof, _drv = struct.unpack_from("<4Q", b, p)
        p += 4 * self.so
        self.root = self._symtab_entry(p)[1]

    # ---------------------------------------------------------------- primitives
    def _o(self, p):
        return struct.unpack_from("<Q" if self.so == 8 else "<I", self.b, p)[0]

    def _l(self, p):
        return struct.unpack_from("<Q" if self.sl == 8 else "<I", self.b, p)[0]

    def _symtab_entry(self, p):
        name_off = self._o(p)
        addr = self._o(p + self.so)
        return name_off, addr

    def _messages(self, addr):
        b = self.b
        if b[addr] != 1:
            raise NotImplementedError("object header v%d" % b[addr])
        nmsg = struct.unpack_from("<H", b, addr + 2)[0]
        hsize = struct.unpack_from("<I", b, addr + 8)[0]
        blocks = [(addr + 16, hsize)]
        out = []
        while blocks and len(out) < nmsg:
            start, size = blocks.pop(0)
            p = start
            while p + 8 <= start + size and len(out) < nmsg:
                mtype, msize, flags = struct.unpack_from("<HHB", b, p)
                data = p + 8
                out.append((mtype, data, msize))
                if mtype == 0x10:
                    blocks.append((self._o(data), self._l(data + self.so)))
                p = data + msize
        return out

    def _heap_name(self, heap_addr, off):
        b = self.b
        assert b[heap_addr:heap_addr + 4] == b"HEAP"
        data = self._o(heap_addr + 8 + 2 * self.sl)
        end = b.index(b"\x00", data + off)
        return b[data + off:end].decode()

    # ---------------------------------------------------------------- groups
    def _group_entries(self, addr):
        for mtype, p, _ in self._messages(addr):
            if mtype == 0x11:
                btree, heap = self._o(p), self._o(p + self.so)
                return self._walk_group_btree(btree, heap)
        raise NotImplementedError("group without symbol table message")

    def _walk_group_btree(self, addr, heap):
        b = self.b
        assert b[addr:addr + 4] == b"TREE", "group b-tree"
        level = b[addr + 5]
        used = struct.unpack_from("<H", b, addr + 6)[0]
        p = addr + 8 + 2 * self.so
        res = {}
        p += self.sl                                   # key 0
        for _ in range(used):
            child = self._o(p); p += self.so
            p += self.sl
            if level > 0:
                res.update(self._walk_group_btree(child, heap))
            else:
                assert b[child:child + 4] == b"SNOD"
                n = struct.unpack_from("<H", b, child + 6)[0]
                q = child + 8
                for _ in range(n):
                    name_off, oh = self._symtab_entry(q)
                    res[self._heap_name(heap, name_off)] = oh
                    q += 2 * self.so + 24
        return res

    def lookup(self, path):
        addr = self.root
        for part in [x for x in path.split("/") if x]:
            addr = self._group_entries(addr)[part]
        return addr

    def keys(self, path="/"):
        return sorted(self._group_entries(self.lookup(path)))

    # ---------------------------------------------------------------- datatypes
    def _dtype(self, p):
        """numpy dtype of the datatype message at p and its encoded size."""
        b = self.b
        cls, ver = b[p] & 0x0F, b[p] >> 4
        bits = b[p + 1] | (b[p + 2] << 8)
        esize = struct.unpack_from("<I", b, p + 4)[0]
        order = ">" if bits & 1 else "<"
        if cls == 1:
            return np.dtype(order + {4: "f4", 8: "f8"}[esize]), 20
        if cls == 0:
            return np.dtype(order + ("i" if bits & 8 else "u") + str(esize)), 12
        if cls == 3:
            return np.dtype("S%d" % esize), 8
        if cls == 6:
            q, fields = p + 8, []
            for _ in range(bits & 0xFFFF):
                e = b.index(b"\0", q)
                name = b[q:e].decode()
                if ver == 1:
                    q = q + ((e - q) // 8 + 1) * 8
                    off = struct.unpack_from("<I", b, q)[0]
                    q += 32
                else:
                    q = e + 1
                    nb = 1 if esize < 256 else 2 if esize < 65536 else 4
                    off = int.from_bytes(b[q:q + nb], "little")
                    q += nb
                mdt, msz = self._dtype(q)
                q += msz
                fields.append((name, mdt, off))
            return np.dtype({"names": [f[0] for f in fields], "formats": [f[1] for f in fields],
                             "offsets": [f[2] for f in fields], "itemsize": esize}), q - p
        if cls == 9:                              # variable length: data in the global heap
            return None, 8
        raise NotImplementedError("datatype class %d" % cls)

    def attrs(self, path="/"):
        """Attributes (version-1 messages) of an object: name -> numpy value or str."""
        b = self.b
        out = {}
        for mtype, p, size in self._messages(self.lookup(path)):
            if mtype != 0x0C or b[p] != 1:
                continue
            nsz, dsz, ssz = struct.unpack_from("<HHH", b, p + 2)
            q = p + 8
            name = b[q:q + nsz - 1].decode()
            q += (nsz + 7) // 8 * 8
            dt, _ = self._dtype(q)
            q += (dsz + 7) // 8 * 8
            if dt is None:
                out[name] = None
                continue
            rank = b[q + 1]
            shape = tuple(self._l(q + 8 + 8 * i) for i in range(rank))
            q += (ssz + 7) // 8 * 8
            n = int(np.prod(shape)) if shape else 1
            v = np.frombuffer(b[q:q + n * dt.itemsize], dtype=dt).reshape(shape)
            out[name] = v.item().rstrip(b"\0").decode() if dt.kind == "S" and not shape else v.copy()
        return out

    # ---------------------------------------------------------------- datasets
    def read(self, path):
        b = self.b
        msgs = self._messages(self.lookup(path))
        shape = dtype = layout = None
        filters = []
        for mtype, p, size in msgs:
            if mtype == 0x01:
                ver, rank, flags = b[p], b[p + 1], b[p + 2]
                q = p + (8 if ver == 1 else 4)
                shape = tuple(self._l(q + i * self.sl) for i in range(rank))
            elif mtype == 0x03:
                dtype, _ = self._dtype(p)
            elif mtype == 0x08:
                ver = b[p]
                if ver == 3:
                    cls = b[p + 1]
                    if cls == 0:
                        n = struct.unpack_from("<H", b, p + 2)[0]
                        layout = ("compact", p + 4, n)
                    elif cls == 1:
                        layout = ("contig", self._o(p + 2), self._l(p + 2 + self.so))
                    else:
                        nd = b[p + 2]
                        bt = self._o(p + 3)
                        cd = struct.unpack_from("<%dI" % nd, b, p + 3 + self.so)
                        layout = ("chunked", bt, cd)
                else:
                    raise NotImplementedError("layout v%d" % ver)
            elif mtype == 0x0B:
                ver, nf = b[p], b[p + 1]
                q = p + (8 if ver == 1 else 2)
                for _ in range(nf):
                    fid = struct.unpack_from("<H", b, q)[0]
                    if ver == 1 or fid >= 256:
                        nlen = struct.unpack_from("<H", b, q + 2)[0]
                        flg, nv = struct.unpack_from("<HH", b, q + 4)
                        q += 8
                        if ver == 1:
                            q += (nlen + 7) // 8 * 8
                        else:
                            q += nlen
                    else:
                        flg, nv = struct.unpack_from("<HH", b, q + 2)
                        q += 6
                    vals = struct.unpack_from("<%dI" % nv, b, q)
                    q += 4 * nv
                    if ver == 1 and nv % 2:
                        q += 4
                    filters.append((fid, vals))
        n = int(np.prod(shape)) if shape else 1
        if layout[0] == "contig":
            raw = b[layout[1]:layout[1] + n * dtype.itemsize]
            return np.frombuffer(raw, dtype=dtype).reshape(shape).copy()
        if layout[0] == "compact":
            return np.frombuffer(b[layout[1]:layout[1] + layout[2]], dtype=dtype)[:n].reshape(shape).copy()
        out = np.zeros(shape, dtype=dtype)
        chunk = layout[2][:-1]
        for offs, caddr, csize, fmask in self._chunks(layout[1], len(shape)):
            data = b[caddr:caddr + csize]
            for i, (fid, vals) in reversed(list(enumerate(filters))):
                if fmask & (1 << i):
                    continue
                if fid == 3:
                    data = data[:-4]
                elif fid == 1:
                    data = zlib.decompress(data)
                elif fid == 2:
                    es = vals[0] if vals else dtype.itemsize
                    a = np.frombuffer(data, dtype=np.uint8)
                    m = len(a) // es
                    data = a[:m * es].reshape(es, m).T.copy().tobytes() + bytes(a[m * es:])
                else:
                    raise NotImplementedError("filter %d" % fid)
            arr = np.frombuffer(data, dtype=dtype)[:int(np.prod(chunk))].reshape(chunk)
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, chunk, shape))
            out[sl] = arr[tuple(slice(0, x.stop - x.start) for x in sl)]
        return out

    def _chunks(self, addr, rank):
        b = self.b
        assert b[addr:addr + 4] == b"TREE", "chunk b-tree"
        level = b[addr + 5]
        used = struct.unpack_from("<H", b, addr + 6)[0]
        p = addr + 8 + 2 * self.so
        ksz = 8 + 8 * (rank + 1)
        for _ in range(used):
            csize, fmask = struct.unpack_from("<II", b, p)
            offs = struct.unpack_from("<%dQ" % rank, b, p + 8)
            child = self._o(p + ksz)
            if level > 0:
                yield from self._chunks(child, rank)
            else:
                yield offs, child, csize, fmask
            p += ksz + self.so
