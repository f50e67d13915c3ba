"""A small reader written from the HDF5 file-format specification (version 0 superblock,
version 1 object headers, symbol-table groups, contiguous datasets): the structures an HDF5
library such as h5py walks to open the files the engine writes.  It shares no code with the
engine's own reader, so a file both accept follows the format rather than one implementation.
"""
from __future__ import annotations

import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class Spec:
    def __init__(self, path):
        self.b = open(path, "rb").read()
        b = self.b
        assert b[:8] == SIGNATURE, "superblock signature"
        assert b[8] == 0, "superblock version 0"
        self.so, self.sl = b[13], b[14]
        assert (self.so, self.sl) == (8, 8), "8-byte offsets and lengths"
        self.leaf_k, self.int_k = struct.unpack_from("<HH", b, 16)
        base, _free, self.eof, _drv = struct.unpack_from("<QQQQ", b, 24)
        assert base == 0
        assert self.eof == len(b), "end-of-file address equals the file size"
        # root group symbol table entry at 56
        _name, self.root_oh, cache = struct.unpack_from("<QQI", b, 56)
        assert cache == 1, "root entry caches its symbol table"
        self.btree, self.heap = struct.unpack_from("<QQ", b, 56 + 24)
        # the root object header's symbol table message (what a library reads) agrees
        stab = [m for t, _f, m in self.messages(self.root_oh) if t == 0x0011]
        assert len(stab) == 1 and struct.unpack_from("<QQ", stab[0], 0) == (self.btree, self.heap), "root symbol table"

    def messages(self, addr):
        """Messages of a version-1 object header: [(type, flags, bytes)]."""
        b = self.b
        ver, _r, nmsg, _refs, size = struct.unpack_from("<BBHII", b, addr)
        assert ver == 1, "object header version 1"
        p, end, out = addr + 16, addr + 16 + size, []
        while len(out) < nmsg and p < end:
            mtype, msize, mflags = struct.unpack_from("<HHB", b, p)
            out.append((mtype, mflags, b[p + 8: p + 8 + msize]))
            p += 8 + msize
        assert len(out) == nmsg, "message count"
        return out

    def heap_string(self, off):
        b = self.b
        assert b[self.heap:self.heap + 4] == b"HEAP"
        size, _free, data = struct.unpack_from("<QQQ", b, self.heap + 8)
        assert off < size
        end = b.index(b"\0", data + off)
        return b[data + off:end].decode()

    def entries(self):
        """name -> object header address, walking the group B-tree and its symbol nodes."""
        b, out = self.b, {}
        stack = [self.btree]
        while stack:
            a = stack.pop()
            assert b[a:a + 4] == b"TREE", "B-tree node"
            ntype, level, used = struct.unpack_from("<BBH", b, a + 4)
            assert ntype == 0, "group node"
            p = a + 8 + 16  # siblings
            assert used <= 2 * self.int_k, "B-tree node within the superblock's 2K capacity"
            for q in range(used):
                child = struct.unpack_from("<Q", b, p + 8)[0]
                p += 16
                if level > 0:
                    stack.append(child)
                    continue
                assert b[child:child + 4] == b"SNOD", "symbol table node"
                nsym = struct.unpack_from("<H", b, child + 6)[0]
                assert nsym <= 2 * self.leaf_k, "symbol node within the superblock's 2K capacity"
                for s in range(nsym):
                    e = child + 8 + 40 * s
                    name_off, oh = struct.unpack_from("<QQ", b, e)
                    out[self.heap_string(name_off)] = oh
        return out

    def dataset(self, name):
        oh = self.entries()[name]
        shape = dtype = data = None
        for mtype, _flags, m in self.messages(oh):
            if mtype == 0x0001:  # dataspace
                ver, rank = m[0], m[1]
                assert ver == 1
                shape = struct.unpack_from("<" + "Q" * rank, m, 8)
            elif mtype == 0x0003:  # datatype
                cls, ver = m[0] & 0x0F, m[0] >> 4
                assert cls == 1 and ver == 1, "IEEE float, datatype version 1"
                size = struct.unpack_from("<I", m, 4)[0]
                little = (m[1] & 1) == 0
                off, prec, epos, esize, mpos, msize, bias = struct.unpack_from("<HHBBBBI", m, 8)
                assert little and off == 0
                assert (size, prec, epos, esize, mpos, msize, bias) in ((8, 64, 52, 11, 0, 52, 1023), (4, 32, 23, 8, 0, 23, 127))
                dtype = "<f8" if size == 8 else "<f4"
            elif mtype == 0x0008:  # data layout
                assert m[0] == 3 and m[1] == 1, "layout version 3, contiguous"
                addr, nbytes = struct.unpack_from("<QQ", m, 2)
                data = (addr, nbytes)
        assert shape is not None and dtype is not None and data is not None
        addr, nbytes = data
        n = int(np.prod(shape))
        assert nbytes == n * np.dtype(dtype).itemsize
        return np.frombuffer(self.b, dtype=dtype, count=n, offset=addr).reshape(shape)
