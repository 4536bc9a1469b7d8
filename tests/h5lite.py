"""Minimal reader for the HDF5 files the sLapH reference writes.

The reference writes one file per diagram through the HDF5 C++ API
(include/h5-wrapper.hpp:106-200): superblock version 0, a root group held as a
version-1 B-tree of symbol-table nodes, and one 1-D dataset of compound
{re: f64, im: f64} per correlator (src/h5-wrapper.cpp:18-26).  No HDF5 library
is available here, so this module walks exactly that subset of the format
(HDF5 file format specification, "Disk Format Level 0/1/2"): superblock v0,
B-tree v1 group nodes, SNOD symbol-table nodes, local heaps, version-1 object
headers with continuation messages, dataspace, compound datatype and
contiguous / compact data layout messages.
"""
from __future__ import annotations

import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(RuntimeError):
    pass


class _File:
    def __init__(self, data: bytes):
        self.b = data
        if data[:8] != b"\x89HDF\r\n\x1a\n":
            raise H5Error("not an HDF5 file")
        if data[8] != 0:
            raise H5Error(f"superblock version {data[8]} not supported")
        self.so = data[13]  # size of offsets
        self.sl = data[14]  # size of lengths
        if self.so != 8 or self.sl != 8:
            raise H5Error("only 8-byte offsets/lengths supported")
        # base addr, free-space addr, eof addr, driver addr: 4 x 8 bytes from 24
        root = 24 + 4 * 8
        self.root_header = self.u64(root + 8)
        cache_type = self.u32(root + 16)
        if cache_type != 1:
            raise H5Error("root entry carries no symbol-table scratch pad")
        self.root_btree = self.u64(root + 24)
        self.root_heap = self.u64(root + 32)

    def u8(self, o):
        return self.b[o]

    def u16(self, o):
        return struct.unpack_from("<H", self.b, o)[0]

    def u32(self, o):
        return struct.unpack_from("<I", self.b, o)[0]

    def u64(self, o):
        return struct.unpack_from("<Q", self.b, o)[0]

    def heap_data(self, heap_addr):
        if self.b[heap_addr:heap_addr + 4] != b"HEAP":
            raise H5Error("bad local heap signature")
        return self.u64(heap_addr + 24)

    def cstr(self, o):
        e = self.b.index(b"\x00", o)
        return self.b[o:e].decode()

    def group_entries(self, btree, heap):
        """(name, object header address) of every link in a v1 group B-tree."""
        data = self.heap_data(heap)
        out = []

        def walk(node):
            if self.b[node:node + 4] != b"TREE":
                raise H5Error("bad B-tree signature")
            if self.u8(node + 4) != 0:
                raise H5Error("not a group B-tree")
            level = self.u8(node + 5)
            used = self.u16(node + 6)
            p = node + 8 + 16  # skip siblings
            p += 8  # key 0
            for _ in range(used):
                child = self.u64(p)
                p += 8 + 8  # child + next key
                if level > 0:
                    walk(child)
                else:
                    snod(child)

        def snod(addr):
            if self.b[addr:addr + 4] != b"SNOD":
                raise H5Error("bad symbol table node signature")
            n = self.u16(addr + 6)
            p = addr + 8
            for _ in range(n):
                name_off = self.u64(p)
                hdr = self.u64(p + 8)
                out.append((self.cstr(data + name_off), hdr))
                p += 40

        walk(btree)
        return out

    def messages(self, hdr):
        """(type, data offset, size) of every message of a v1 object header."""
        if self.u8(hdr) != 1:
            raise H5Error("only version-1 object headers supported")
        nmsg = self.u16(hdr + 2)
        size = self.u32(hdr + 8)
        blocks = [(hdr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            p = start
            while p + 8 <= start + length and len(out) < nmsg:
                mtype = self.u16(p)
                msize = self.u16(p + 2)
                body = p + 8
                if mtype == 0x10:  # continuation
                    blocks.append((self.u64(body), self.u64(body + 8)))
                out.append((mtype, body, msize))
                p = body + msize
        return out

    def dataset(self, hdr):
        dims = None
        dtype = None
        layout = None
        for mtype, body, msize in self.messages(hdr):
            if mtype == 0x1:  # dataspace
                ver = self.u8(body)
                ndim = self.u8(body + 1)
                if ver == 1:
                    p = body + 8
                elif ver == 2:
                    p = body + 4
                else:
                    raise H5Error("dataspace version")
                dims = tuple(self.u64(p + 8 * i) for i in range(ndim))
            elif mtype == 0x3:  # datatype
                cls_ver = self.u8(body)
                cls = cls_ver & 0x0F
                tsize = self.u32(body + 4)
                if cls != 6 or tsize != 16:
                    raise H5Error("expected a 16-byte compound type")
                names = []
                p = body + 8
                nmemb = self.u16(body + 1)
                for _ in range(nmemb):
                    nm = self.cstr(p)
                    names.append(nm)
                    p += (len(nm) + 1 + 7) // 8 * 8
                    off = self.u32(p)
                    p += 4 + 1 + 3 + 4 + 4 + 16  # v1 member: offset, dims, reserved, perm, dim sizes
                    # member datatype: class/version(1) bits(3) size(4) + properties
                    mcls = self.u8(p) & 0x0F
                    if mcls != 1:
                        raise H5Error("compound member is not floating point")
                    p += 8 + 12  # float properties
                    if (nm, off) not in (("re", 0), ("im", 8)):
                        raise H5Error(f"unexpected member {nm}@{off}")
                dtype = names
            elif mtype == 0x8:  # layout
                ver = self.u8(body)
                if ver != 3:
                    raise H5Error("layout version")
                cls = self.u8(body + 1)
                if cls == 1:
                    layout = ("contiguous", self.u64(body + 2), self.u64(body + 10))
                elif cls == 0:
                    n = self.u16(body + 2)
                    layout = ("compact", body + 4, n)
                else:
                    raise H5Error("chunked layout not supported")
        if dims is None or dtype is None or layout is None:
            raise H5Error("incomplete dataset header")
        n = int(np.prod(dims)) if dims else 1
        _, addr, size = layout
        if addr == UNDEF:
            return np.zeros(n, dtype=np.complex128)
        if size < 16 * n:
            raise H5Error("dataset storage too small")
        arr = np.frombuffer(self.b, dtype="<f8", count=2 * n, offset=addr)
        return (arr[0::2] + 1j * arr[1::2]).astype(np.complex128)


def read_correlators(path) -> dict[str, np.ndarray]:
    """All datasets of a reference correlator file as {name: complex array}."""
    with open(path, "rb") as f:
        data = f.read()
    h5 = _File(data)
    out = {}
    for name, hdr in h5.group_entries(h5.root_btree, h5.root_heap):
        out[name] = h5.dataset(hdr)
    return out
