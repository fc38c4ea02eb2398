"""A small writer of MATLAB v7.3-style MAT-files (HDF5 behind MATLAB's 512-byte
header), test infrastructure for sid_gb300.matfile: superblock version 0,
a root group stored as a symbol table (B-tree version 1, one SNOD, a local
heap), datasets with version-1 object headers, contiguous layout or chunked
layout (B-tree version 1) with the deflate filter.  Arrays are given in
MATLAB's shape and written the way MATLAB does: the dataspace holds the
dimensions reversed and the data in column-major order."""
import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


def _pad8(b):
    return b + b"\x00" * (-len(b) % 8)


def _msg(mtype, body):
    body = _pad8(body)
    return struct.pack("<HHB3x", mtype, len(body), 0) + body


def _obj_header(msgs):
    data = b"".join(msgs)
    return struct.pack("<BBHII", 1, 0, len(msgs), 1, len(data)) + b"\x00" * 4 + data


def _datatype(dt):
    dt = np.dtype(dt)
    if dt.kind == "f":
        if dt.itemsize == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            sign = 31
        else:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            sign = 63
        return bytes([0x11, 0x20, sign, 0]) + struct.pack("<I", dt.itemsize) + props
    signed = 0x08 if dt.kind == "i" else 0
    return bytes([0x10, signed, 0, 0]) + struct.pack("<I", dt.itemsize) + struct.pack("<HH", 0, 8 * dt.itemsize)


def _dataspace(dims):
    return struct.pack("<BBB5x", 1, len(dims), 0) + b"".join(struct.pack("<Q", d) for d in dims)


class _File:
    def __init__(self):
        self.buf = bytearray()

    def alloc(self, data):
        data = _pad8(bytes(data))
        addr = len(self.buf)
        self.buf += data
        return addr

    def reserve(self, n):
        addr = len(self.buf)
        self.buf += b"\x00" * (n + (-n % 8))
        return addr

    def put(self, addr, data):
        self.buf[addr:addr + len(data)] = data


def write_mat73(path, variables, chunks=None, deflate=6):
    """variables: {name: array (MATLAB shape)}; chunks: {name: chunk shape in
    MATLAB order} for chunked + deflate storage, others contiguous."""
    chunks = chunks or {}
    f = _File()
    sb_addr = f.reserve(96)  # superblock (addresses are relative to it: base address = 512)
    names = sorted(variables)
    heap_data = b"\x00" * 8
    name_off = {}
    for n in names:
        name_off[n] = len(heap_data)
        heap_data += _pad8(n.encode() + b"\x00")
    objs = {}
    for n in names:
        a = np.asarray(variables[n])
        if a.ndim == 0:
            a = a.reshape(1, 1)
        raw_dims = tuple(reversed(a.shape))
        cdata = np.ascontiguousarray(a.T)  # C-order data of the reversed dims = MATLAB column-major
        msgs = [_msg(0x01, _dataspace(raw_dims)), _msg(0x03, _datatype(a.dtype))]
        if n in chunks:
            cm = tuple(reversed(chunks[n]))
            grid = [int(np.ceil(d / c)) for d, c in zip(raw_dims, cm)]
            entries = []
            for idx in np.ndindex(*grid):
                off = [i * c for i, c in zip(idx, cm)]
                blk = np.zeros(cm, dtype=a.dtype)
                sl = tuple(slice(o, min(o + c, d)) for o, c, d in zip(off, cm, raw_dims))
                blk[tuple(slice(0, s.stop - s.start) for s in sl)] = cdata[sl]
                comp = zlib.compress(blk.tobytes(), deflate)
                entries.append((off, f.alloc(comp), len(comp)))
            nk = len(raw_dims) + 1
            node = b"TREE" + struct.pack("<BBHQQ", 1, 0, len(entries), UNDEF, UNDEF)
            for off, addr, size in entries:
                node += struct.pack("<II", size, 0) + b"".join(struct.pack("<Q", o) for o in off + [0])
                node += struct.pack("<Q", addr)
            node += struct.pack("<II", 0, 0) + b"".join(struct.pack("<Q", d) for d in list(raw_dims) + [0])
            bt = f.alloc(node)
            layout = struct.pack("<BBBQ", 3, 2, nk, bt) + b"".join(struct.pack("<I", c) for c in cm) + \
                struct.pack("<I", a.dtype.itemsize)
            filt = struct.pack("<BB6x", 1, 1) + struct.pack("<HHHH", 1, 0, 0, 1) + struct.pack("<I", deflate) + \
                b"\x00" * 4
            msgs += [_msg(0x08, layout), _msg(0x0B, filt)]
        else:
            daddr = f.alloc(cdata.tobytes())
            msgs.append(_msg(0x08, struct.pack("<BBQQ", 3, 1, daddr, cdata.nbytes)))
        objs[n] = f.alloc(_obj_header(msgs))
    heap_addr = f.reserve(32)
    heap_data_addr = f.alloc(heap_data)
    f.put(heap_addr, b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), UNDEF, heap_data_addr))
    snod = b"SNOD" + struct.pack("<BBH", 1, 0, len(names))
    for n in names:
        snod += struct.pack("<QQII", name_off[n], objs[n], 0, 0) + b"\x00" * 16
    snod_addr = f.alloc(snod)
    btree = b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, UNDEF, UNDEF) + struct.pack("<QQQ", 0, snod_addr,
                                                                                  name_off[names[-1]])
    bt_addr = f.alloc(btree)
    root = f.alloc(_obj_header([_msg(0x11, struct.pack("<QQ", bt_addr, heap_addr))]))
    eof = len(f.buf)
    sb = b"\x89HDF\r\n\x1a\n" + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0)
    sb += struct.pack("<QQQQ", 512, UNDEF, eof, UNDEF)
    sb += struct.pack("<QQII", 0, root, 1, 0) + struct.pack("<QQ", bt_addr, heap_addr)
    f.put(sb_addr, sb)
    header = b"MATLAB 7.3 MAT-file, written for tests" + b" " * 200
    header = header[:116] + b"\x00" * 8 + struct.pack("<H", 0x0200) + b"IM"
    header = header + b"\x00" * (512 - len(header))
    with open(path, "wb") as fh:
        fh.write(header)
        fh.write(bytes(f.buf))
