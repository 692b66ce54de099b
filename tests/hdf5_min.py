"""A reader for the subset of HDF5 that TimeEvolver's result files use (TEST
INFRASTRUCTURE ONLY; no HDF5 library exists on either machine).

It follows the published HDF5 file-format specification (version 0 superblock,
version 1 object headers, symbol-table groups with a version 1 B-tree and a
local heap) and understands the messages the reference's ``saveResult``
produces (helper/krylovHelper.cpp:27-92 through the HDF5 C++ API): dataspace,
datatype (IEEE float and two's-complement integer, little endian), fill value,
contiguous layout, attribute, modification time, object header continuation
and symbol table.  Anything else raises, so a file that parses here uses only
those structures.  ``read(path)`` returns ``{name: (array, {attr: value})}``
for the datasets of the root group, in link order.
"""
import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class FormatError(ValueError):
    pass


def _u(buf, off, n):
    return int.from_bytes(buf[off:off + n], "little")


class _File:
    def __init__(self, raw):
        self.raw = raw
        if raw[:8] != SIGNATURE:
            raise FormatError("no HDF5 signature")
        if raw[8] != 0:
            raise FormatError("superblock version %d (only 0)" % raw[8])
        self.so, self.sl = raw[13], raw[14]
        if (self.so, self.sl) != (8, 8):
            raise FormatError("offset/length sizes %d/%d" % (self.so, self.sl))
        self.leaf_k = _u(raw, 16, 2)
        self.internal_k = _u(raw, 18, 2)
        base, fsa, eof, drv = (_u(raw, 24 + 8 * i, 8) for i in range(4))
        if base != 0 or fsa != UNDEF or drv != UNDEF:
            raise FormatError("unexpected base/free-space/driver addresses")
        if eof != len(raw):
            raise FormatError("end-of-file address %d, file size %d" % (eof, len(raw)))
        self.eof = eof
        # root group symbol table entry at 56
        self.root_header = _u(raw, 64, 8)
        cache = _u(raw, 72, 4)
        if cache != 1:
            raise FormatError("root entry cache type %d" % cache)
        self.root_btree, self.root_heap = _u(raw, 80, 8), _u(raw, 88, 8)

    # ---------------------------------------------------------------- heaps
    def local_heap(self, addr):
        r = self.raw
        if r[addr:addr + 4] != b"HEAP" or r[addr + 4] != 0:
            raise FormatError("local heap at %d" % addr)
        size = _u(r, addr + 8, 8)
        data = _u(r, addr + 24, 8)
        return r[data:data + size]

    @staticmethod
    def heap_string(heap, off):
        end = heap.index(b"\0", off)
        return heap[off:end].decode()

    # ---------------------------------------------------------- B-tree (groups)
    def group_entries(self, btree, heap_addr):
        heap = self.local_heap(heap_addr)
        out = []
        self._walk(btree, heap, out)
        return out

    def _walk(self, addr, heap, out):
        r = self.raw
        if r[addr:addr + 4] != b"TREE":
            raise FormatError("B-tree node at %d" % addr)
        if r[addr + 4] != 0:
            raise FormatError("B-tree node type %d (only group nodes)" % r[addr + 4])
        level = r[addr + 5]
        used = _u(r, addr + 6, 2)
        p = addr + 24
        for i in range(used):
            p += 8  # key (heap offset)
            child = _u(r, p, 8)
            p += 8
            if level > 0:
                self._walk(child, heap, out)
            else:
                self._snod(child, heap, out)

    def _snod(self, addr, heap, out):
        r = self.raw
        if r[addr:addr + 4] != b"SNOD" or r[addr + 4] != 1:
            raise FormatError("symbol table node at %d" % addr)
        count = _u(r, addr + 6, 2)
        p = addr + 8
        for i in range(count):
            name_off, header = _u(r, p, 8), _u(r, p + 8, 8)
            out.append((self.heap_string(heap, name_off), header))
            p += 40

    # -------------------------------------------------------- object headers
    def messages(self, addr):
        r = self.raw
        if r[addr] != 1:
            raise FormatError("object header version %d at %d" % (r[addr], addr))
        nmsg = _u(r, addr + 2, 2)
        size = _u(r, addr + 8, 4)
        blocks = [(addr + 16, size)]
        msgs = []
        while blocks:
            start, length = blocks.pop(0)
            p, end = start, start + length
            while p < end and len(msgs) < nmsg:
                mtype, msize, flags = _u(r, p, 2), _u(r, p + 2, 2), r[p + 4]
                body = r[p + 8:p + 8 + msize]
                if msize % 8:
                    raise FormatError("message size %d not a multiple of 8" % msize)
                if mtype == 0x10:
                    blocks.append((_u(body, 0, 8), _u(body, 8, 8)))
                msgs.append((mtype, flags, body))
                p += 8 + msize
        if len(msgs) != nmsg:
            raise FormatError("object header at %d: %d of %d messages" % (addr, len(msgs), nmsg))
        return msgs

    # ------------------------------------------------------------- messages
    @staticmethod
    def dataspace(body):
        ver, rank, flags = body[0], body[1], body[2]
        if ver != 1:
            raise FormatError("dataspace version %d" % ver)
        dims = [_u(body, 8 + 8 * i, 8) for i in range(rank)]
        return tuple(dims)

    @staticmethod
    def datatype(body):
        cls_ver = body[0]
        cls, ver = cls_ver & 0x0F, cls_ver >> 4
        if ver != 1:
            raise FormatError("datatype version %d" % ver)
        bits0 = body[1]
        size = _u(body, 4, 4)
        if bits0 & 1:
            raise FormatError("big-endian datatype")
        if cls == 1:  # floating point
            if size == 8:
                return np.dtype("<f8")
            if size == 4:
                return np.dtype("<f4")
        elif cls == 0:  # fixed point
            signed = bool(bits0 & 0x08)
            return np.dtype(("<i%d" if signed else "<u%d") % size)
        raise FormatError("datatype class %d size %d" % (cls, size))

    @staticmethod
    def layout(body):
        ver = body[0]
        if ver != 3 or body[1] != 1:
            raise FormatError("layout version %d class %d (only contiguous v3)" % (ver, body[1]))
        return _u(body, 2, 8), _u(body, 10, 8)

    def attribute(self, body):
        ver = body[0]
        if ver != 1:
            raise FormatError("attribute version %d" % ver)
        nsz, tsz, ssz = _u(body, 2, 2), _u(body, 4, 2), _u(body, 6, 2)
        p = 8
        name = body[p:p + nsz].split(b"\0")[0].decode()
        p += (nsz + 7) // 8 * 8
        dt = self.datatype(body[p:p + tsz])
        p += (tsz + 7) // 8 * 8
        dims = self.dataspace(body[p:p + ssz])
        p += (ssz + 7) // 8 * 8
        count = int(np.prod(dims)) if dims else 1
        val = np.frombuffer(body[p:p + count * dt.itemsize], dtype=dt).copy()
        return name, val

    def dataset(self, addr):
        dims = dt = lay = None
        attrs = {}
        kinds = []
        for mtype, flags, body in self.messages(addr):
            kinds.append(mtype)
            if mtype == 0x01:
                dims = self.dataspace(body)
            elif mtype == 0x03:
                dt = self.datatype(body)
            elif mtype == 0x08:
                lay = self.layout(body)
            elif mtype == 0x0C:
                name, val = self.attribute(body)
                attrs[name] = val
            elif mtype in (0x00, 0x05, 0x10, 0x12):
                pass
            else:
                raise FormatError("message type %#x" % mtype)
        if dims is None or dt is None or lay is None:
            raise FormatError("object at %d is not a dataset" % addr)
        a, size = lay
        count = int(np.prod(dims))
        if size != count * dt.itemsize or a + size > self.eof:
            raise FormatError("dataset storage out of range")
        arr = np.frombuffer(self.raw[a:a + size], dtype=dt).copy().reshape(dims)
        return arr, attrs, kinds, a


def read(path, with_layout=False):
    """Datasets of the root group: {name: (array, {attr: np.array})}; with
    with_layout, also the message types and the data address of each."""
    raw = open(path, "rb").read()
    f = _File(raw)
    root = f.messages(f.root_header)
    stab = [b for t, _, b in root if t == 0x11]
    if len(stab) != 1:
        raise FormatError("root group without a symbol table message")
    bt, hp = _u(stab[0], 0, 8), _u(stab[0], 8, 8)
    if (bt, hp) != (f.root_btree, f.root_heap):
        raise FormatError("root symbol table differs from the superblock's cache")
    out = {}
    for name, hdr in f.group_entries(bt, hp):
        arr, attrs, kinds, addr = f.dataset(hdr)
        out[name] = (arr, attrs, kinds, addr) if with_layout else (arr, attrs)
    return out
