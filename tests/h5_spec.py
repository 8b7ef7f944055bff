"""A second, independent reader of the HDF5 structures the results files use
(test infrastructure): superblock versions 0/1 (after a user block too),
version-1 object headers with continuation blocks, symbol-table groups
(version-1 B-tree, local heap, symbol-table nodes), dataspace versions 1/2,
float / integer / fixed-string datatypes, layouts versions 1-3 (contiguous,
compact) and attribute messages versions 1-3, written from the published
file format. Besides reading, it checks the index invariants a library
lookup relies on: names sorted within and across symbol-table nodes, each
B-tree key the last name of its child, key 0 the empty name, and every node
allocated at the full size its K values imply.
"""
from __future__ import annotations

import struct

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = (1 << 64) - 1


class H5Spec:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        at = 0
        while at + 8 <= len(self.b):
            if self.b[at:at + 8] == SIG:
                break
            at = 512 if at == 0 else 2 * at
        else:
            raise ValueError("no superblock")
        sb = self.b[at:]
        ver = sb[8]
        assert ver in (0, 1), ver
        assert sb[13] == 8 and sb[14] == 8
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", sb, 16)
        p = 24 + (4 if ver == 1 else 0)
        self.base, self.freespace, self.eof, self.driver = struct.unpack_from("<4Q", sb, p)
        self.root = struct.unpack_from("<Q", sb, p + 32 + 8)[0]
        self.root_cache = struct.unpack_from("<QQ", sb, p + 32 + 24) if struct.unpack_from("<I", sb, p + 32 + 16)[0] == 1 else None

    def at(self, addr, n):
        a = self.base + addr
        assert addr != UNDEF and a + n <= len(self.b), (addr, n)
        return self.b[a:a + n]

    # ---- object headers
    def messages(self, addr):
        pre = self.at(addr, 16)
        assert pre[0] == 1, "object header version"
        nmsgs, = struct.unpack_from("<H", pre, 2)
        chunk, = struct.unpack_from("<I", pre, 8)
        chunks = [(addr + 16, chunk)]
        out, seen = [], 0
        while chunks:
            a, n = chunks.pop(0)
            d = self.at(a, n)
            p = 0
            while p + 8 <= len(d) and seen < nmsgs:
                typ, size, flags = struct.unpack_from("<HHB", d, p)
                body = d[p + 8:p + 8 + size]
                assert len(body) == size
                seen += 1
                if typ == 0x10:
                    chunks.append(struct.unpack_from("<QQ", body, 0))
                elif typ != 0:
                    out.append((typ, flags, body))
                p += 8 + size
        assert seen == nmsgs, (seen, nmsgs)
        return out

    # ---- groups
    def members(self, addr, check=True):
        stab = [m for m in self.messages(addr) if m[0] == 0x11]
        assert stab, "not a symbol-table group"
        bt, hp = struct.unpack_from("<QQ", stab[0][2], 0)
        h = self.at(hp, 32)
        assert h[:4] == b"HEAP" and h[4] == 0
        dsize, free, daddr = struct.unpack_from("<3Q", h, 8)
        assert free == 1 or free < dsize, "bad heap free list"
        heap = self.at(daddr, dsize)
        name = lambda off: heap[off:heap.index(b"\0", off)].decode()  # noqa: E731
        out = []
        self._walk(bt, name, out, check)
        if check:
            names = [n for n, _ in out]
            assert names == sorted(names, key=lambda s: s.encode()), names
        return out

    def _walk(self, addr, name, out, check):
        node_bytes = 24 + (2 * self.internal_k + 1) * 8 + 2 * self.internal_k * 8
        h = self.at(addr, node_bytes if check else 24)
        assert h[:4] == b"TREE" and h[4] == 0
        level, used = h[5], struct.unpack_from("<H", h, 6)[0]
        kc = self.at(addr + 24, (2 * used + 1) * 8)
        keys = [struct.unpack_from("<Q", kc, 16 * i)[0] for i in range(used + 1)]
        kids = [struct.unpack_from("<Q", kc, 8 + 16 * i)[0] for i in range(used)]
        if check:
            assert name(keys[0]) == "" or level > 0
        for i, c in enumerate(kids):
            start = len(out)
            if level > 0:
                self._walk(c, name, out, check)
            else:
                snod_bytes = 8 + 2 * self.leaf_k * 40
                s = self.at(c, snod_bytes if check else 8)
                assert s[:4] == b"SNOD" and s[4] == 1
                nsym, = struct.unpack_from("<H", s, 6)
                e = self.at(c + 8, 40 * nsym)
                for j in range(nsym):
                    off, oh = struct.unpack_from("<QQ", e, 40 * j)
                    out.append((name(off), oh))
            if check and len(out) > start:
                assert name(keys[i + 1]) == out[-1][0], (name(keys[i + 1]), out[-1][0])

    def resolve(self, path):
        addr = self.root
        for part in [p for p in path.split("/") if p]:
            addr = dict(self.members(addr))[part]
        return addr

    def is_group(self, addr):
        return any(m[0] == 0x11 for m in self.messages(addr))

    # ---- values
    @staticmethod
    def _dspace(d):
        ver, rank = d[0], d[1]
        if ver == 1:
            p = 8
        else:
            assert ver == 2
            if d[3] == 2:
                return []
            p = 4
        return list(struct.unpack_from(f"<{rank}Q", d, p))

    @staticmethod
    def _decode(dt, raw, count):
        cls, size = dt[0] & 0x0F, struct.unpack_from("<I", dt, 4)[0]
        be = dt[1] & 1
        e = ">" if be else "<"
        if cls == 1:
            return list(struct.unpack(e + ("d" if size == 8 else "f") * count, raw[:size * count]))
        if cls == 0:
            code = {1: "b", 2: "h", 4: "i", 8: "q"}[size]
            if not dt[1] & 0x08:
                code = code.upper()
            return list(struct.unpack(e + code * count, raw[:size * count]))
        if cls == 3:
            return raw[:size * count].split(b"\0")[0].decode()
        raise ValueError(f"class {cls}")

    def dataset(self, path):
        msgs = {m[0]: m[2] for m in self.messages(self.resolve(path))}
        dims = self._dspace(msgs[0x1])
        dt = msgs[0x3]
        size = struct.unpack_from("<I", dt, 4)[0]
        count = 1
        for d in dims:
            count *= d
        lay = msgs[0x8]
        if lay[0] == 3:
            if lay[1] == 1:
                addr, nbytes = struct.unpack_from("<QQ", lay, 2)
                assert nbytes == count * size
                raw = bytes(count * size) if addr == UNDEF else self.at(addr, count * size)
            else:
                assert lay[1] == 0
                raw = lay[4:4 + count * size]
        else:
            dimsz, cls = lay[1], lay[2]
            if cls == 1:
                addr, = struct.unpack_from("<Q", lay, 8)
                raw = self.at(addr, count * size)
            else:
                raw = lay[8 + 4 * dimsz + 4:]
        return dims, self._decode(dt, raw, count)

    def attrs(self, path):
        out = {}
        for typ, _, m in self.messages(self.resolve(path)):
            if typ != 0xC:
                continue
            ver = m[0]
            nl, tl, sl = struct.unpack_from("<HHH", m, 2)
            p = 9 if ver == 3 else 8
            pad = (lambda n: (n + 7) & ~7) if ver == 1 else (lambda n: n)
            name = m[p:p + nl].split(b"\0")[0].decode()
            p += pad(nl)
            dt = m[p:p + tl]
            p += pad(tl)
            ds = m[p:p + sl]
            p += pad(sl)
            dims = [] if ds[1] == 0 else self._dspace(ds)
            count = 1
            for d in dims:
                count *= d
            out[name] = self._decode(dt, m[p:], count)
        return out
