"""A small HDF5 reader written from the published HDF5 file-format specification
(superblock versions 0-1, symbol-table groups, version-1 object headers,
contiguous, compact and chunked datasets with the deflate filter).

Test infrastructure only: it checks the files written by the run driver's
HDF5 writer.  The reader itself is checked against HDF5 files written by the
HDF5 library (tests/test_h5.py).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(Exception):
    pass


class Dataset:
    def __init__(self, f: "H5File", name: str, msgs: list):
        self.name = name
        self.f = f
        self.shape = None
        self.maxshape = None
        self.dtype = None
        self.layout = None
        self.filters = []
        self.fill = None
        self.messages = [m[0] for m in msgs]
        for mtype, body in msgs:
            if mtype == 0x0001:
                self.shape, self.maxshape = f._dataspace(body)
            elif mtype == 0x0003:
                self.dtype = f._datatype(body)
            elif mtype == 0x0008:
                self.layout = f._layout(body)
            elif mtype == 0x000B:
                self.filters = f._filters(body)
            elif mtype == 0x0005:
                self.fill = body

    def read(self) -> np.ndarray:
        f, kind = self.f, self.layout[0]
        n = int(np.prod(self.shape)) if self.shape else 1
        if kind == "contiguous":
            addr, size = self.layout[1], self.layout[2]
            if addr == UNDEF:
                return np.zeros(self.shape, self.dtype)
            if len(self.layout) == 4 and len(self.layout[3]) == len(self.shape):
                size *= self.dtype.itemsize      # version 1-2 layout: dims without the element size
            if size < n * self.dtype.itemsize:
                raise H5Error(f"{self.name}: contiguous storage of {size} B for {n} elements")
            return np.frombuffer(f.buf, self.dtype, n, addr).reshape(self.shape).copy()
        if kind == "compact":
            return np.frombuffer(self.layout[1], self.dtype, n).reshape(self.shape).copy()
        # chunked: walk the version-1 B-tree of type 1
        btree, cdims = self.layout[1], self.layout[2]
        out = np.zeros(self.shape, self.dtype)
        rank = len(self.shape)
        for offs, csize, mask in f._chunks(btree, rank):
            raw = f.buf[offs[0]:offs[0] + csize]
            for fid in reversed(self.filters):
                if mask & (1 << self.filters.index(fid)):
                    continue
                if fid == 1:
                    raw = zlib.decompress(raw)
                elif fid == 2:      # shuffle
                    a = np.frombuffer(raw, np.uint8).reshape(self.dtype.itemsize, -1)
                    raw = a.T.tobytes()
                else:
                    raise H5Error(f"filter {fid} not supported")
            chunk = np.frombuffer(raw, self.dtype, int(np.prod(cdims[:rank]))).reshape(cdims[:rank])
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs[1], cdims, self.shape))
            out[sl] = chunk[tuple(slice(0, x.stop - x.start) for x in sl)]
        return out


class H5File:
    def __init__(self, path):
        self.buf = open(path, "rb").read()
        b = self.buf
        base = None
        for off in (0, 512, 1024, 2048, 4096, 8192):
            if b[off:off + 8] == SIGNATURE:
                base = off
                break
        if base is None:
            raise H5Error("no HDF5 signature")
        self.base = base
        ver = b[base + 8]
        if ver not in (0, 1):
            raise H5Error(f"superblock version {ver} not supported")
        self.superblock_version = ver
        self.O, self.L = b[base + 13], b[base + 14]
        if (self.O, self.L) != (8, 8):
            raise H5Error("only 8-byte offsets and lengths")
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", b, base + 16)
        p = base + 24 + (4 if ver == 1 else 0)
        self.base_addr, self.freespace, self.eof, self.driver = struct.unpack_from("<4Q", b, p)
        p += 32
        self.root_entry = self._entry(p)
        if self.base_addr != base:
            raise H5Error("base address differs from the signature offset")

    # ---- primitive structures -------------------------------------------------
    def _entry(self, p):
        name_off, ohdr, cache, _ = struct.unpack_from("<QQII", self.buf, p)
        scratch = self.buf[p + 24:p + 40]
        return dict(name_off=name_off, ohdr=ohdr, cache=cache, scratch=scratch)

    def _addr(self, a):
        return a + self.base if a != UNDEF else a

    def _heap(self, addr):
        b = self.buf
        p = self._addr(addr)
        if b[p:p + 4] != b"HEAP":
            raise H5Error("local heap signature")
        size, free, data = struct.unpack_from("<QQQ", b, p + 8)
        data = self._addr(data)
        # the free list: offsets inside the data segment, ended by 1 (as the library writes it)
        seen = 0
        while free != 1:
            if free == UNDEF or free + 16 > size or seen > size:
                raise H5Error("bad local heap free list")
            free, fsize = struct.unpack_from("<QQ", b, data + free)
            if fsize < 16:
                raise H5Error("bad local heap free block")
            seen += 1
        return data, size

    def _heap_str(self, heap, off):
        data, size = heap
        if off >= size:
            raise H5Error("heap offset out of range")
        end = self.buf.index(b"\0", data + off)
        return self.buf[data + off:end].decode()

    def _messages(self, addr):
        """All messages of a version-1 object header (continuations followed)."""
        b = self.buf
        p = self._addr(addr)
        if b[p] == ord("O") and b[p:p + 4] == b"OHDR":
            raise H5Error("version-2 object headers not supported")
        ver, _, nmsg, refc, size = struct.unpack_from("<BBHII", b, p)
        if ver != 1:
            raise H5Error(f"object header version {ver}")
        blocks = [(p + 16, size)]
        msgs = []
        while blocks and len(msgs) < nmsg:
            q, size = blocks.pop(0)
            end = q + size
            while q + 8 <= end and len(msgs) < nmsg:
                mtype, msize, flags = struct.unpack_from("<HHB", b, q)
                body = b[q + 8:q + 8 + msize]
                if q + 8 + msize > end:
                    raise H5Error("message runs past its header block")
                if mtype == 0x0010:
                    caddr, clen = struct.unpack_from("<QQ", body)
                    blocks.append((self._addr(caddr), clen))
                msgs.append((mtype, body))
                q += 8 + msize
        return msgs

    def _dataspace(self, body):
        ver, rank, flags = body[0], body[1], body[2]
        if ver == 1:
            p = 8
        elif ver == 2:
            p = 4
        else:
            raise H5Error(f"dataspace version {ver}")
        dims = struct.unpack_from(f"<{rank}Q", body, p)
        p += 8 * rank
        maxd = struct.unpack_from(f"<{rank}Q", body, p) if flags & 1 else dims
        return tuple(dims), tuple(maxd)

    def _datatype(self, body):
        cls, ver = body[0] & 0x0F, body[0] >> 4
        bits = body[1] | (body[2] << 8) | (body[3] << 16)
        size = struct.unpack_from("<I", body, 4)[0]
        order = ">" if bits & 1 else "<"
        if cls == 1:
            return np.dtype(f"{order}f{size}")
        if cls == 0:
            return np.dtype(f"{order}{'i' if bits & 8 else 'u'}{size}")
        raise H5Error(f"datatype class {cls} not supported")

    def _layout(self, body):
        ver = body[0]
        if ver == 3:
            cls = body[1]
            if cls == 1:
                addr, size = struct.unpack_from("<QQ", body, 2)
                return ("contiguous", self._addr(addr), size)
            if cls == 0:
                n = struct.unpack_from("<H", body, 2)[0]
                return ("compact", body[4:4 + n])
            if cls == 2:
                rank = body[2]
                addr = struct.unpack_from("<Q", body, 3)[0]
                dims = struct.unpack_from(f"<{rank}I", body, 11)
                return ("chunked", addr, dims)
        if ver in (1, 2):
            rank, cls = body[1], body[2]
            p = 8
            if cls == 0:
                dims = struct.unpack_from(f"<{rank}I", body, p)
                p += 4 * rank
                n = struct.unpack_from("<I", body, p)[0]
                return ("compact", body[p + 4:p + 4 + n])
            addr = struct.unpack_from("<Q", body, p)[0]
            dims = struct.unpack_from(f"<{rank}I", body, p + 8)
            if cls == 1:
                return ("contiguous", self._addr(addr), int(np.prod(dims, dtype=np.int64)), dims)
            return ("chunked", addr, dims)
        raise H5Error(f"layout message version {ver}")

    def _filters(self, body):
        ver, n = body[0], body[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = struct.unpack_from("<H", body, p)[0]
            if ver == 1 or fid >= 256:
                nlen = struct.unpack_from("<H", body, p + 2)[0]
            else:
                nlen = 0
            flags, ncv = struct.unpack_from("<HH", body, p + (4 if (ver == 1 or fid >= 256) else 2))
            p += (8 if (ver == 1 or fid >= 256) else 6)
            if nlen:
                p += (nlen + 7) // 8 * 8 if ver == 1 else nlen
            p += 4 * ncv
            if ver == 1 and ncv % 2:
                p += 4
            out.append(fid)
        return out

    def _chunks(self, addr, rank):
        b = self.buf
        p = self._addr(addr)
        if b[p:p + 4] != b"TREE":
            raise H5Error("chunk B-tree signature")
        ntype, level, used = b[p + 4], b[p + 5], struct.unpack_from("<H", b, p + 6)[0]
        if ntype != 1:
            raise H5Error("not a chunk B-tree")
        q = p + 24
        ksize = 8 + 8 * (rank + 1)
        for i in range(used):
            csize, mask = struct.unpack_from("<II", b, q)
            offs = struct.unpack_from(f"<{rank}Q", b, q + 8)
            child = struct.unpack_from("<Q", b, q + ksize)[0]
            q += ksize + 8
            if level == 0:
                yield (self._addr(child), offs), csize, mask
            else:
                yield from self._chunks(child, rank)

    def _group_entries(self, btree, heap_addr):
        """(name, object header address) of a symbol-table group, in B-tree order."""
        b = self.buf
        heap = self._heap(heap_addr)
        out = []

        def walk(addr):
            p = self._addr(addr)
            if b[p:p + 4] != b"TREE":
                raise H5Error("group B-tree signature")
            ntype, level, used = b[p + 4], b[p + 5], struct.unpack_from("<H", b, p + 6)[0]
            if ntype != 0:
                raise H5Error("not a group B-tree")
            q = p + 24
            keys, kids = [], []
            for i in range(used):
                keys.append(struct.unpack_from("<Q", b, q)[0])
                kids.append(struct.unpack_from("<Q", b, q + 8)[0])
                q += 16
            keys.append(struct.unpack_from("<Q", b, q)[0])
            prev = self._heap_str(heap, keys[0])
            for i, c in enumerate(kids):
                if level > 0:
                    walk(c)
                    continue
                s = self._addr(c)
                if b[s:s + 4] != b"SNOD":
                    raise H5Error("symbol node signature")
                nsym = struct.unpack_from("<H", b, s + 6)[0]
                if nsym > 2 * self.leaf_k:
                    raise H5Error("symbol node holds more than 2K entries")
                names = []
                for j in range(nsym):
                    e = self._entry(s + 8 + 40 * j)
                    names.append(self._heap_str(heap, e["name_off"]))
                    out.append((names[-1], e["ohdr"]))
                if names != sorted(names, key=lambda x: x.encode()):
                    raise H5Error("symbol node entries not in name order")
                hi = self._heap_str(heap, keys[i + 1])
                if names and not (prev.encode() < names[0].encode() and names[-1].encode() <= hi.encode()):
                    raise H5Error("B-tree keys do not bound the symbol node")
                prev = hi

        walk(btree)
        return out

    # ---- public ---------------------------------------------------------------
    def root_messages(self):
        return self._messages(self.root_entry["ohdr"])

    def datasets(self) -> dict:
        """name -> Dataset for every dataset in the root group."""
        stab = [m for m in self.root_messages() if m[0] == 0x0011]
        if not stab:
            raise H5Error("root group has no symbol table message")
        btree, heap = struct.unpack_from("<QQ", stab[0][1])
        if self.root_entry["cache"] == 1:
            sb, sh = struct.unpack_from("<QQ", self.root_entry["scratch"])
            if (sb, sh) != (btree, heap):
                raise H5Error("root scratch pad disagrees with the symbol table message")
        out = {}
        for name, addr in self._group_entries(btree, heap):
            msgs = self._messages(addr)
            if any(m[0] == 0x0008 for m in msgs):
                out[name] = Dataset(self, name, msgs)
        return out
