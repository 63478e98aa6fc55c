"""A second, independent reading of the HDF5 file-format specification, used only by the tests.

It walks a file with a version-0 superblock the way the specification lays it out (superblock, root
symbol-table entry, root object header, local heap, group B-tree, symbol-table nodes, dataset object
headers) and returns every structure it passed through, so that tests can check both the values and
the layout rules (signatures, sizes, sort order, B-tree keys, the end-of-file address). It is checked
against a file written by the HDF5 library itself before it is used on the library's own files.
"""
from __future__ import annotations

import struct

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5File:
    def __init__(self, blob: bytes):
        self.b = blob
        self.sb = next(off for off in [0] + [512 << k for k in range(20)]
                       if off + 8 <= len(blob) and blob[off:off + 8] == SIGNATURE)
        b = blob[self.sb:]
        self.version = b[8]
        assert self.version == 0, "version-0 superblock expected"
        self.size_offsets, self.size_lengths = b[13], b[14]
        assert (self.size_offsets, self.size_lengths) == (8, 8)
        self.leaf_k, self.internal_k, self.flags = struct.unpack("<HHI", b[16:24])
        self.base, self.freespace, self.eof, self.driver = struct.unpack("<QQQQ", b[24:56])
        self.root_entry = self._entry(self.sb + 56)
        self.datasets: dict[str, dict] = {}
        self.heap_names: list[str] = []
        self._walk_root()

    def _at(self, addr: int) -> int:
        return self.base + addr

    def _entry(self, off: int) -> dict:
        name_off, header, cache, _ = struct.unpack("<QQII", self.b[off:off + 24])
        s0, s1 = struct.unpack("<QQ", self.b[off + 24:off + 40])
        return dict(name_off=name_off, header=header, cache=cache, scratch=(s0, s1))

    def messages(self, addr: int) -> list[tuple[int, int, bytes]]:
        p = self._at(addr)
        version, _, nmsgs, refcount, size = struct.unpack("<BBHII", self.b[p:p + 12])
        assert version == 1 and refcount >= 1
        out, q, end = [], p + 16, p + 16 + size
        while q < end and len(out) < nmsgs:
            mtype, msize, flags = struct.unpack("<HHB", self.b[q:q + 5])
            assert msize % 8 == 0, "message sizes are multiples of 8 in version-1 headers"
            out.append((mtype, flags, self.b[q + 8:q + 8 + msize]))
            q += 8 + msize
        assert len(out) == nmsgs
        return out

    def _walk_root(self) -> None:
        msgs = self.messages(self.root_entry["header"])
        (btree, heap), = [struct.unpack("<QQ", d[:16]) for t, _, d in msgs if t == 0x0011]
        self.btree_addr, self.heap_addr = btree, heap
        p = self._at(heap)
        assert self.b[p:p + 4] == b"HEAP" and self.b[p + 4] == 0
        self.heap_size, self.heap_free, data = struct.unpack("<QQQ", self.b[p + 8:p + 32])
        self.heap = self.b[self._at(data):self._at(data) + self.heap_size]
        self._walk_btree(btree)

    def name_at(self, off: int) -> str:
        return self.heap[off:self.heap.index(b"\0", off)].decode()

    def _walk_btree(self, addr: int) -> None:
        p = self._at(addr)
        assert self.b[p:p + 4] == b"TREE" and self.b[p + 4] == 0
        level, used = self.b[p + 5], struct.unpack("<H", self.b[p + 6:p + 8])[0]
        vals = struct.unpack(f"<{2 * used + 1}Q", self.b[p + 24:p + 24 + 8 * (2 * used + 1)])
        keys, children = vals[0::2], vals[1::2]
        self.btree_keys = list(keys)
        for i, child in enumerate(children):
            if level:
                self._walk_btree(child)
                continue
            q = self._at(child)
            assert self.b[q:q + 4] == b"SNOD" and self.b[q + 4] == 1
            n = struct.unpack("<H", self.b[q + 6:q + 8])[0]
            names = []
            for e in range(n):
                ent = self._entry(q + 8 + 40 * e)
                name = self.name_at(ent["name_off"])
                names.append(name)
                self.datasets[name] = self._dataset(ent["header"])
            assert names == sorted(names, key=lambda s: s.encode()), "symbol-table entries in strcmp order"
            assert self.name_at(keys[i + 1]) == names[-1], "B-tree key i+1 names the last entry of child i"
            self.heap_names += names

    def _dataset(self, addr: int) -> dict:
        ds = {"header": addr}
        for t, flags, d in self.messages(addr):
            if t == 0x0001:
                version, rank = d[0], d[1]
                first = 8 if version == 1 else 4
                ds["shape"] = struct.unpack(f"<{rank}Q", d[first:first + 8 * rank])
            elif t == 0x0003:
                ds["dtype"] = d[:20]
                ds["elem"] = struct.unpack("<I", d[4:8])[0]
            elif t == 0x0005:
                ds["fill"] = d
            elif t == 0x0008:
                if d[0] == 3:
                    assert d[1] == 1, "contiguous"
                    ds["addr"], ds["nbytes"] = struct.unpack("<QQ", d[2:18])
                else:
                    assert d[2] == 1, "contiguous"
                    ds["addr"] = struct.unpack("<Q", d[8:16])[0]
        return ds

    def read(self, name: str):
        import numpy as np
        ds = self.datasets[name]
        count = int(np.prod(ds["shape"])) if ds["shape"] else 1
        p = self._at(ds["addr"])
        fmt = "<f8" if ds["elem"] == 8 else "<f4"
        return np.frombuffer(self.b[p:p + count * ds["elem"]], dtype=fmt).astype(np.float64).reshape(ds["shape"])
