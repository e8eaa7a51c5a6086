"""A reader for the subset of HDF5 that libsgdg's vlasov.h5 writer produces
(version 0 superblock, old-style root group, contiguous 64-bit datasets),
written from the HDF5 File Format Specification and checking, besides the
values, every structural field a library reader relies on: signatures,
versions, sizes, the end-of-file address, the local heap's free list, the
B-tree node and symbol table node sizes implied by the superblock's K values,
and the name order of the symbol table.  Test infrastructure only."""
import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(AssertionError):
    pass


def _need(cond, what):
    if not cond:
        raise H5Error(what)


def _u(buf, off, n):
    return int.from_bytes(buf[off:off + n], "little")


def _object_header(buf, addr):
    """Messages of a version 1 object header: list of (type, flags, data)."""
    _need(buf[addr] == 1, "object header version 1")
    nmsg = _u(buf, addr + 2, 2)
    _need(_u(buf, addr + 4, 4) >= 1, "reference count")
    size = _u(buf, addr + 8, 4)
    _need(size % 8 == 0, "object header size multiple of 8")
    p, end = addr + 16, addr + 16 + size
    msgs = []
    while p < end:
        mtype, msize, flags = _u(buf, p, 2), _u(buf, p + 2, 2), buf[p + 4]
        _need(msize % 8 == 0, "message size padded to 8")
        msgs.append((mtype, flags, bytes(buf[p + 8:p + 8 + msize])))
        p += 8 + msize
    _need(p == end and len(msgs) == nmsg, "message count and object header size agree")
    return msgs


def _dataset(buf, addr, eof):
    msgs = {t: (f, d) for t, f, d in _object_header(buf, addr)}
    _need(set(msgs) >= {0x0001, 0x0003, 0x0008}, "dataspace, datatype and layout messages")
    _, ds = msgs[0x0001]
    _need(ds[0] == 1 and ds[2] == 0, "dataspace version 1 without maximum sizes")
    rank = ds[1]
    dims = [_u(ds, 8 + 8 * i, 8) for i in range(rank)]
    _, dt = msgs[0x0003]
    cls, ver = dt[0] & 0x0F, dt[0] >> 4
    _need(ver == 1 and _u(dt, 4, 4) == 8, "datatype version 1, 8 bytes")
    if cls == 0:
        _need(dt[1] == 0x08 and _u(dt, 8, 2) == 0 and _u(dt, 10, 2) == 64, "signed 64-bit little-endian integer")
        dtype = np.dtype("<i8")
    else:
        _need(cls == 1, "fixed or floating point")
        _need(bytes(dt[1:4]) == b"\x20\x3f\x00" and _u(dt, 8, 2) == 0 and _u(dt, 10, 2) == 64
              and tuple(dt[12:16]) == (52, 11, 0, 52) and _u(dt, 16, 4) == 1023, "IEEE 754 double, little endian")
        dtype = np.dtype("<f8")
    if 0x0005 in msgs:
        _, fv = msgs[0x0005]
        _need(fv[0] == 2 and fv[1] in (1, 2, 3) and fv[2] in (0, 1, 2), "fill value version 2")
    _, lay = msgs[0x0008]
    _need(lay[0] == 3 and lay[1] == 1, "layout version 3, contiguous")
    daddr, dsize = _u(lay, 2, 8), _u(lay, 10, 8)
    count = int(np.prod(dims)) if rank else 1
    _need(dsize == 8 * count, "layout size = elements x 8")
    if dsize == 0:
        return np.zeros(0, dtype)
    _need(daddr != UNDEF and daddr + dsize <= eof, "data inside the file")
    a = np.frombuffer(buf, dtype, count, daddr).copy()
    return a if rank else a[0]


def read(path):
    """{name: value} of the root group's datasets (scalars as numpy scalars)."""
    buf = memoryview(open(path, "rb").read())
    _need(bytes(buf[:8]) == b"\x89HDF\r\n\x1a\n", "signature")
    _need(tuple(buf[8:16]) == (0, 0, 0, 0, 0, 8, 8, 0), "superblock version 0, 8-byte offsets and lengths")
    leafk, intk = _u(buf, 16, 2), _u(buf, 18, 2)
    _need(leafk > 0 and intk > 0, "K values")
    _need(_u(buf, 24, 8) == 0 and _u(buf, 32, 8) == UNDEF and _u(buf, 48, 8) == UNDEF, "base, free space, driver")
    eof = _u(buf, 40, 8)
    _need(eof == len(buf), "end-of-file address = file size")
    root = 56
    _need(_u(buf, root, 8) == 0 and _u(buf, root + 16, 4) == 1, "root entry caches the symbol table")
    root_oh, btree, heap = _u(buf, root + 8, 8), _u(buf, root + 24, 8), _u(buf, root + 32, 8)
    msgs = _object_header(buf, root_oh)
    _need(len(msgs) == 1 and msgs[0][0] == 0x0011, "root group: one symbol table message")
    _need((_u(msgs[0][2], 0, 8), _u(msgs[0][2], 8, 8)) == (btree, heap), "symbol table message = root scratch pad")
    # local heap
    _need(bytes(buf[heap:heap + 4]) == b"HEAP" and buf[heap + 4] == 0, "local heap version 0")
    hsize, hfree, hdata = _u(buf, heap + 8, 8), _u(buf, heap + 16, 8), _u(buf, heap + 24, 8)
    _need(hsize % 8 == 0 and hdata + hsize <= eof, "heap data segment")
    _need(buf[hdata] == 0, "heap offset 0 holds the empty name")
    f = hfree
    while f != 1:  # free list: 1 ends it
        _need(f % 8 == 0 and f + 16 <= hsize, "free block inside the heap")
        nxt, size = _u(buf, hdata + f, 8), _u(buf, hdata + f + 8, 8)
        _need(size >= 16 and f + size <= hsize, "free block size")
        f = nxt

    def name_at(off):
        _need(off < hsize, "name offset inside the heap")
        e = bytes(buf[hdata + off:hdata + hsize]).index(b"\0")
        return bytes(buf[hdata + off:hdata + off + e]).decode()

    # group B-tree (leaf level): children are symbol table nodes
    _need(bytes(buf[btree:btree + 4]) == b"TREE" and buf[btree + 4] == 0, "group B-tree node")
    _need(buf[btree + 5] == 0, "B-tree of one leaf level")
    used = _u(buf, btree + 6, 2)
    _need(1 <= used <= 2 * intk, "children within 2K")
    _need(btree + 24 + (2 * intk + 1) * 8 + 2 * intk * 8 <= eof, "B-tree node sized for 2K children")
    out, names = {}, []
    for c in range(used):
        key_lo = _u(buf, btree + 24 + 16 * c, 8)
        snod = _u(buf, btree + 32 + 16 * c, 8)
        key_hi = _u(buf, btree + 40 + 16 * c, 8)
        _need(bytes(buf[snod:snod + 4]) == b"SNOD" and buf[snod + 4] == 1, "symbol table node version 1")
        nsym = _u(buf, snod + 6, 2)
        _need(nsym <= 2 * leafk and snod + 8 + 2 * leafk * 40 <= eof, "symbol table node sized for 2K entries")
        child = []
        for i in range(nsym):
            e = snod + 8 + 40 * i
            nm = name_at(_u(buf, e, 8))
            _need(_u(buf, e + 16, 4) == 0, "dataset entries cache nothing")
            child.append(nm)
            out[nm] = _dataset(buf, _u(buf, e + 8, 8), eof)
        _need(not child or name_at(key_hi) == child[-1], "right key = last name of the child")
        _need(c > 0 or name_at(key_lo) == "", "left key of the first child = empty name")
        names += child
    enc = [n.encode() for n in names]
    _need(enc == sorted(enc) and len(set(enc)) == len(enc), "names unique and in byte order")
    return out
