"""Minimal reader of the HDF5 files that hold pylbm's golden results.

TEST INFRASTRUCTURE ONLY, used by make_demo_golden.py to turn the reference's
``tests/reference/*.h5`` files into npz fixtures (h5py is not available).

Handles exactly what those files use, written by h5py through
pylbm/hdf5.py:204-206: superblock version 0, a root group with an old-style
symbol table (v1 B-tree of group nodes and a local heap), and datasets of
little-endian IEEE floats stored contiguously.  Layout of every structure is
the one of the published HDF5 file-format specification (superblock v0,
symbol table entry, object header v1, messages 0x0001 dataspace, 0x0003
datatype, 0x0008 data layout, 0x0010 continuation, 0x0011 symbol table).
"""
import struct

import numpy as np

_SIGNATURE = b"\x89HDF\r\n\x1a\n"


class H5Error(ValueError):
    pass


class _File:
    def __init__(self, data):
        if data[:8] != _SIGNATURE:
            raise H5Error("not an HDF5 file")
        if data[8] != 0:
            raise H5Error(f"superblock version {data[8]} is not supported")
        self.d = data
        self.so, self.sl = data[13], data[14]
        if self.so != 8 or self.sl != 8:
            raise H5Error("only 8-byte offsets and lengths are supported")
        # superblock v0: 24 bytes of versions and sizes, 4 addresses, root entry
        self.root_entry = 24 + 4 * self.so

    def u(self, off, n):
        return int.from_bytes(self.d[off:off + n], "little")

    # ---------------------------------------------------------------- groups
    def entry(self, off):
        """Symbol table entry: (name offset, object header address, cache type, scratch)."""
        return (self.u(off, 8), self.u(off + 8, 8), self.u(off + 16, 4), self.d[off + 24:off + 40])

    def heap_name(self, heap, offset):
        if self.d[heap:heap + 4] != b"HEAP":
            raise H5Error("bad local heap")
        seg = self.u(heap + 8 + 2 * self.sl, self.so)
        end = self.d.index(b"\0", seg + offset)
        return self.d[seg + offset:end].decode()

    def group_entries(self, btree, heap):
        """(name, header address) of every link of a v1 group B-tree."""
        out = []
        if self.d[btree:btree + 4] != b"TREE":
            raise H5Error("bad group B-tree")
        level = self.d[btree + 5]
        used = self.u(btree + 6, 2)
        p = btree + 8 + 2 * self.so  # first key
        children = []
        for _ in range(used):
            p += self.sl              # key
            children.append(self.u(p, self.so))
            p += self.so
        for child in children:
            if level > 0:
                out += self.group_entries(child, heap)
                continue
            if self.d[child:child + 4] != b"SNOD":
                raise H5Error("bad symbol table node")
            nsym = self.u(child + 6, 2)
            for i in range(nsym):
                name_off, header, _, _ = self.entry(child + 8 + 40 * i)
                out.append((self.heap_name(heap, name_off), header))
        return out

    # ---------------------------------------------------------------- headers
    def messages(self, header):
        """(type, data offset, size) of every message of a version-1 object header."""
        if self.d[header] != 1:
            raise H5Error(f"object header version {self.d[header]} is not supported")
        nmsg = self.u(header + 2, 2)
        blocks = [(header + 16, self.u(header + 8, 4))]
        out = []
        while blocks and len(out) < nmsg:
            start, size = blocks.pop(0)
            p = start
            while p + 8 <= start + size and len(out) < nmsg:
                mtype, msize = self.u(p, 2), self.u(p + 2, 2)
                out.append((mtype, p + 8, msize))
                if mtype == 0x0010:  # continuation block
                    blocks.append((self.u(p + 8, self.so), self.u(p + 8 + self.so, self.sl)))
                p += 8 + msize
        return out

    def dataset(self, header):
        dims = dtype = addr = None
        for mtype, p, size in self.messages(header):
            if mtype == 0x0001:  # dataspace
                version, rank = self.d[p], self.d[p + 1]
                first = p + (8 if version == 1 else 4)
                dims = [self.u(first + 8 * i, 8) for i in range(rank)]
            elif mtype == 0x0003:  # datatype
                cls, bits, nbytes = self.d[p] & 0x0F, self.d[p + 1], self.u(p + 4, 4)
                if cls != 1 or bits & 1:
                    raise H5Error("only little-endian floating point datasets are supported")
                dtype = {4: "<f4", 8: "<f8"}[nbytes]
            elif mtype == 0x0008:  # data layout
                version = self.d[p]
                if version == 3:
                    if self.d[p + 1] != 1:
                        raise H5Error("only contiguous datasets are supported")
                    addr = self.u(p + 2, self.so)
                else:
                    if self.d[p + 2] != 1:
                        raise H5Error("only contiguous datasets are supported")
                    addr = self.u(p + 8, self.so)
        if dims is None or dtype is None or addr is None:
            raise H5Error("incomplete dataset header")
        count = int(np.prod(dims)) if dims else 1
        return np.frombuffer(self.d, dtype=dtype, count=count, offset=addr).reshape(dims).copy()


def read(path):
    """All datasets of the root group: {name: ndarray}."""
    with open(path, "rb") as fh:
        f = _File(fh.read())
    _, header, cache, scratch = f.entry(f.root_entry)
    if cache == 1:
        btree, heap = struct.unpack("<QQ", scratch)
    else:
        btree = heap = None
        for mtype, p, _ in f.messages(header):
            if mtype == 0x0011:
                btree, heap = f.u(p, 8), f.u(p + 8, 8)
        if btree is None:
            raise H5Error("root group without a symbol table")
    return {name: f.dataset(addr) for name, addr in f.group_entries(btree, heap)}
