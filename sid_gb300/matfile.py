"""MATLAB v7.3 MAT-files (HDF5) without an HDF5 library: the PSF file of SID.

sid_main.m:30 opens the PSF with ``matfile`` and reads ``H``
(M x M x Nnum x Nnum x Z), ``Nnum`` and ``CAindex`` (Z x 2); save_psf_fast.m
writes them with ``h5create`` / ``h5write`` into a ``-v7.3`` file, i.e. an
HDF5 file behind MATLAB's 512-byte header.  This module reads the subset of
HDF5 such files use:

* superblock versions 0-3 (the base address of version 0/1 files written
  behind the MATLAB header is 512);
* object headers version 1 and 2 (``OHDR`` / ``OCHK``), with continuation
  blocks;
* groups stored as symbol tables (B-tree version 1 of ``SNOD`` nodes plus a
  local ``HEAP``) or as compact link messages;
* datasets with contiguous, compact or chunked (B-tree version 1) layout
  (layout messages version 1-3),
  the deflate / shuffle / Fletcher-32 filters, little- or big-endian integer
  and IEEE floating-point element types.

HDF5 stores a MATLAB array's dimensions in reverse order (row-major), so an
array read here is transposed back: the result has MATLAB's shape and
Fortran (column-major) order, the layout libsid takes.  A contiguous dataset
is read through a memory map.  Dense (fractal-heap) link storage, variable-
length types, compound types and references are not supported and raise.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"


class MatFileError(ValueError):
    pass


class _H5:
    def __init__(self, path):
        self.path = path
        self.f = open(path, "rb")
        self.sb = self._find_superblock()
        self._parse_superblock()

    # ------------------------------------------------------------- low level
    def close(self):
        self.f.close()

    def read(self, addr, n):
        self.f.seek(self.base + addr)
        b = self.f.read(n)
        if len(b) != n:
            raise MatFileError(f"{self.path}: truncated read at {addr}")
        return b

    def _find_superblock(self):
        for off in (0, 512, 1024, 2048, 4096, 8192, 16384):
            self.f.seek(off)
            if self.f.read(8) == _SIG:
                return off
        raise MatFileError(f"{self.path}: not an HDF5 (MATLAB v7.3) file")

    def _uint(self, b, pos, n):
        return int.from_bytes(b[pos:pos + n], "little"), pos + n

    def _parse_superblock(self):
        self.f.seek(self.sb)
        head = self.f.read(128)
        ver = head[8]
        if ver in (0, 1):
            self.so, self.sl = head[13], head[14]
            pos = 24 + (4 if ver == 1 else 0)
            self.base, pos = self._uint(head, pos, self.so)
            pos += 3 * self.so  # free-space, end-of-file, driver info addresses
            # root group symbol table entry
            _, pos = self._uint(head, pos, self.so)  # link name offset
            self.root, pos = self._uint(head, pos, self.so)
        elif ver in (2, 3):
            self.so, self.sl = head[9], head[10]
            pos = 12
            self.base, pos = self._uint(head, pos, self.so)
            pos += 2 * self.so  # superblock extension, end of file
            self.root, pos = self._uint(head, pos, self.so)
        else:
            raise MatFileError(f"HDF5 superblock version {ver} is not supported")

    # ---------------------------------------------------------- object headers
    def messages(self, addr):
        """[(type, data bytes)] of the object header at addr."""
        b = self.read(addr, 4)
        if b == b"OHDR":
            return self._messages_v2(addr)
        return self._messages_v1(addr)

    def _messages_v1(self, addr):
        h = self.read(addr, 16)
        if h[0] != 1:
            raise MatFileError(f"object header version {h[0]} at {addr}")
        nmsg = int.from_bytes(h[2:4], "little")
        size = int.from_bytes(h[8:12], "little")
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            a, n = blocks.pop(0)
            data = self.read(a, n)
            pos = 0
            while pos + 8 <= n and len(out) < nmsg:
                mtype = int.from_bytes(data[pos:pos + 2], "little")
                msize = int.from_bytes(data[pos + 2:pos + 4], "little")
                body = data[pos + 8:pos + 8 + msize]
                pos += 8 + msize
                if mtype == 0x10:
                    ca, cl = int.from_bytes(body[:self.so], "little"), int.from_bytes(body[self.so:self.so + self.sl],
                                                                                       "little")
                    blocks.append((ca, cl))
                out.append((mtype, body))
        return out

    def _messages_v2(self, addr):
        h = self.read(addr, 16)
        flags = h[5]
        pos = 6
        if flags & 0x20:
            pos += 16
        if flags & 0x10:
            pos += 4
        csz_len = 1 << (flags & 3)
        head = self.read(addr, pos + csz_len)
        size0 = int.from_bytes(head[pos:pos + csz_len], "little")
        blocks = [(addr + pos + csz_len, size0)]
        track = bool(flags & 0x04)
        out = []
        while blocks:
            a, n = blocks.pop(0)
            data = self.read(a, n)
            p = 0
            while p + 4 <= n:
                mtype = data[p]
                msize = int.from_bytes(data[p + 1:p + 3], "little")
                p += 4 + (2 if track else 0)
                body = data[p:p + msize]
                p += msize
                if mtype == 0 and msize == 0:
                    continue
                if mtype == 0x10:
                    ca = int.from_bytes(body[:self.so], "little")
                    cl = int.from_bytes(body[self.so:self.so + self.sl], "little")
                    if self.read(ca, 4) != b"OCHK":
                        raise MatFileError("bad object header continuation block")
                    blocks.append((ca + 4, cl - 8))  # signature and checksum
                out.append((mtype, body))
        return out

    # ------------------------------------------------------------------ groups
    def group_links(self, addr):
        """{name: object header address} of the group at addr."""
        links = {}
        for mtype, body in self.messages(addr):
            if mtype == 0x11:  # symbol table: B-tree v1 + local heap
                bt = int.from_bytes(body[:self.so], "little")
                heap = int.from_bytes(body[self.so:2 * self.so], "little")
                hdata = self._local_heap(heap)
                self._walk_group_btree(bt, hdata, links)
            elif mtype == 0x06:
                name, target = self._link_message(body)
                if target is not None:
                    links[name] = target
            elif mtype == 0x02:
                fh = int.from_bytes(body[2 + (8 if body[1] & 1 else 0):][:self.so], "little")
                if fh != (1 << (8 * self.so)) - 1:
                    raise MatFileError("groups in dense (fractal heap) link storage are not supported")
        return links

    def _local_heap(self, addr):
        h = self.read(addr, 8 + 2 * self.sl + self.so)
        if h[:4] != b"HEAP":
            raise MatFileError("bad local heap")
        size = int.from_bytes(h[8:8 + self.sl], "little")
        data_addr = int.from_bytes(h[8 + 2 * self.sl:8 + 2 * self.sl + self.so], "little")
        return self.read(data_addr, size)

    @staticmethod
    def _cstr(buf, off):
        end = buf.index(b"\x00", off)
        return buf[off:end].decode("utf-8", "replace")

    def _walk_group_btree(self, addr, heap, links):
        h = self.read(addr, 8 + 2 * self.so)
        if h[:4] != b"TREE":
            raise MatFileError("bad group B-tree node")
        level = h[5]
        used = int.from_bytes(h[6:8], "little")
        body = self.read(addr + 8 + 2 * self.so, (2 * used + 1) * max(self.sl, self.so) + self.so * used)
        pos = self.sl  # key 0
        for _ in range(used):
            child = int.from_bytes(body[pos:pos + self.so], "little")
            pos += self.so + self.sl
            if level > 0:
                self._walk_group_btree(child, heap, links)
            else:
                self._symbol_node(child, heap, links)

    def _symbol_node(self, addr, heap, links):
        h = self.read(addr, 8)
        if h[:4] != b"SNOD":
            raise MatFileError("bad symbol table node")
        n = int.from_bytes(h[6:8], "little")
        esz = 2 * self.so + 24
        data = self.read(addr + 8, n * esz)
        for i in range(n):
            e = data[i * esz:(i + 1) * esz]
            name_off = int.from_bytes(e[:self.so], "little")
            obj = int.from_bytes(e[self.so:2 * self.so], "little")
            links[self._cstr(heap, name_off)] = obj

    def _link_message(self, b):
        flags = b[1]
        pos = 2
        ltype = 0
        if flags & 0x08:
            ltype = b[pos]
            pos += 1
        if flags & 0x04:
            pos += 8
        if flags & 0x10:
            pos += 1
        nlen_size = 1 << (flags & 3)
        nlen = int.from_bytes(b[pos:pos + nlen_size], "little")
        pos += nlen_size
        name = b[pos:pos + nlen].decode("utf-8", "replace")
        pos += nlen
        if ltype != 0:
            return name, None  # soft / external links are not followed
        return name, int.from_bytes(b[pos:pos + self.so], "little")

    # ---------------------------------------------------------------- datasets
    def dataset(self, addr):
        shape = dtype = layout = None
        filters = []
        for mtype, body in self.messages(addr):
            if mtype == 0x01:
                shape = self._dataspace(body)
            elif mtype == 0x03:
                dtype = self._datatype(body)
            elif mtype == 0x08:
                layout = self._layout(body)
            elif mtype == 0x0B:
                filters = self._filters(body)
        if shape is None or dtype is None or layout is None:
            raise MatFileError("object is not a dataset")
        return self._read_data(shape, dtype, layout, filters)

    def _dataspace(self, b):
        ver, nd = b[0], b[1]
        pos = 8 if ver == 1 else 4
        dims = [int.from_bytes(b[pos + i * self.sl:pos + (i + 1) * self.sl], "little") for i in range(nd)]
        return tuple(dims)

    @staticmethod
    def _datatype(b):
        cls = b[0] & 0x0F
        bits = b[1] | (b[2] << 8) | (b[3] << 16)
        size = int.from_bytes(b[4:8], "little")
        order = ">" if bits & 1 else "<"
        if cls == 0:
            signed = bool(bits & 0x08)
            return np.dtype(f"{order}{'i' if signed else 'u'}{size}")
        if cls == 1:
            if size not in (2, 4, 8):
                raise MatFileError(f"floating-point size {size} is not supported")
            return np.dtype(f"{order}f{size}")
        raise MatFileError(f"HDF5 datatype class {cls} is not supported")

    def _layout(self, b):
        ver = b[0]
        if ver in (1, 2):
            # version, dimensionality, class, 5 reserved bytes, [address], dims (4 bytes each)
            nd, cls = b[1], b[2]
            pos = 8
            if cls in (1, 2):
                a = int.from_bytes(b[pos:pos + self.so], "little")
                pos += self.so
            dims = [int.from_bytes(b[pos + 4 * i:pos + 4 * i + 4], "little") for i in range(nd)]
            pos += 4 * nd
            if cls == 0:
                n = int.from_bytes(b[pos:pos + 4], "little")
                return ("compact", b[pos + 4:pos + 4 + n])
            if cls == 1:
                return ("contiguous", a)
            return ("chunked", a, dims)
        if ver != 3:
            raise MatFileError(f"data layout message version {ver} is not supported")
        cls = b[1]
        if cls == 0:
            n = int.from_bytes(b[2:4], "little")
            return ("compact", b[4:4 + n])
        if cls == 1:
            a = int.from_bytes(b[2:2 + self.so], "little")
            return ("contiguous", a)
        if cls == 2:
            nd = b[2]
            bt = int.from_bytes(b[3:3 + self.so], "little")
            pos = 3 + self.so
            cdims = [int.from_bytes(b[pos + 4 * i:pos + 4 * i + 4], "little") for i in range(nd)]
            return ("chunked", bt, cdims)
        raise MatFileError(f"data layout class {cls} is not supported")

    @staticmethod
    def _filters(b):
        ver, n = b[0], b[1]
        pos = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = int.from_bytes(b[pos:pos + 2], "little")
            if ver == 1 or fid >= 256:
                nlen = int.from_bytes(b[pos + 2:pos + 4], "little")
                flags = int.from_bytes(b[pos + 4:pos + 6], "little")
                ncd = int.from_bytes(b[pos + 6:pos + 8], "little")
                pos += 8 + ((nlen + 7) // 8 * 8 if ver == 1 else nlen)
            else:
                flags = int.from_bytes(b[pos + 2:pos + 4], "little")
                ncd = int.from_bytes(b[pos + 4:pos + 6], "little")
                pos += 6
            cd = [int.from_bytes(b[pos + 4 * i:pos + 4 * i + 4], "little") for i in range(ncd)]
            pos += 4 * ncd
            if ver == 1 and ncd % 2:
                pos += 4
            out.append((fid, flags, cd))
        return out

    @staticmethod
    def _unfilter(raw, filters, mask, itemsize):
        for i in range(len(filters) - 1, -1, -1):
            fid, _, cd = filters[i]
            if mask & (1 << i):
                continue
            if fid == 1:
                raw = zlib.decompress(raw)
            elif fid == 2:
                es = cd[0] if cd else itemsize
                a = np.frombuffer(raw, dtype=np.uint8)
                n = a.size // es
                raw = a[:n * es].reshape(es, n).T.tobytes() + a[n * es:].tobytes()
            elif fid == 3:
                raw = raw[:-4]
            else:
                raise MatFileError(f"HDF5 filter {fid} is not supported")
        return raw

    def _read_data(self, shape, dtype, layout, filters):
        n = int(np.prod(shape)) if shape else 1
        if layout[0] == "compact":
            arr = np.frombuffer(layout[1][:n * dtype.itemsize], dtype=dtype).copy()
        elif layout[0] == "contiguous":
            if layout[1] == (1 << (8 * self.so)) - 1:
                arr = np.zeros(n, dtype=dtype)  # never written
            else:
                arr = np.memmap(self.path, dtype=dtype, mode="r", offset=self.base + layout[1], shape=(n,))
        else:
            arr = self._read_chunked(shape, dtype, layout, filters)
        arr = np.asarray(arr).reshape(shape) if shape else np.asarray(arr).reshape(())
        return arr

    def _read_chunked(self, shape, dtype, layout, filters):
        _, bt, cdims = layout
        nd = len(shape)
        cshape = cdims[:nd]
        out = np.zeros(shape, dtype=dtype)
        for offs, size, mask, caddr in self._chunk_entries(bt, nd + 1):
            raw = self._unfilter(self.read(caddr, size), filters, mask, dtype.itemsize)
            block = np.frombuffer(raw, dtype=dtype, count=int(np.prod(cshape))).reshape(cshape)
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs[:nd], cshape, shape))
            out[sl] = block[tuple(slice(0, x.stop - x.start) for x in sl)]
        return out

    def _chunk_entries(self, addr, nk):
        h = self.read(addr, 8 + 2 * self.so)
        if h[:4] != b"TREE" or h[4] != 1:
            raise MatFileError("bad chunk B-tree node")
        level = h[5]
        used = int.from_bytes(h[6:8], "little")
        ksz = 8 + 8 * nk
        body = self.read(addr + 8 + 2 * self.so, (used + 1) * ksz + used * self.so)
        pos = 0
        for _ in range(used):
            size = int.from_bytes(body[pos:pos + 4], "little")
            mask = int.from_bytes(body[pos + 4:pos + 8], "little")
            offs = [int.from_bytes(body[pos + 8 + 8 * i:pos + 16 + 8 * i], "little") for i in range(nk)]
            child = int.from_bytes(body[pos + ksz:pos + ksz + self.so], "little")
            pos += ksz + self.so
            if level > 0:
                yield from self._chunk_entries(child, nk)
            else:
                yield offs, size, mask, child


def matfile_read(path: str, names=None) -> dict:
    """Variables of a MATLAB v7.3 MAT-file as NumPy arrays with MATLAB's shape
    (Fortran order).  names: the variables to read (default all numeric
    datasets at the top level)."""
    h = _H5(path)
    try:
        links = h.group_links(h.root)
        out = {}
        for name, addr in links.items():
            if names is not None and name not in names:
                continue
            try:
                arr = h.dataset(addr)
            except MatFileError:
                if names is not None:
                    raise
                continue
            out[name] = np.asfortranarray(arr.T) if arr.ndim > 1 else np.asarray(arr)
        if names is not None:
            missing = [n for n in names if n not in out]
            if missing:
                raise MatFileError(f"{path}: no variable(s) {missing}")
        return out
    finally:
        h.close()


def load_psf(path: str) -> dict:
    """psf_ballistic = matfile(psffile) (sid_main.m:30): H (M x M x Nnum x Nnum
    x Z, single), Nnum and CAindex (Z x 2, when present) of a PSF file written
    by save_psf_fast.m (or MATLAB's save -v7.3)."""
    h = _H5(path)
    try:
        links = h.group_links(h.root)
    finally:
        h.close()
    want = ["H", "Nnum"] + (["CAindex"] if "CAindex" in links else [])
    v = matfile_read(path, want)
    H = v["H"]
    if H.ndim == 4:
        H = H[..., None]
    if H.ndim != 5 or H.shape[0] != H.shape[1] or H.shape[2] != H.shape[3]:
        raise MatFileError(f"{path}: H must be M x M x Nnum x Nnum x Z, got {H.shape}")
    out = {"H": np.asfortranarray(H, dtype=np.float32), "Nnum": int(np.asarray(v["Nnum"]).ravel()[0])}
    if "CAindex" in v:
        out["CAindex"] = np.asfortranarray(np.asarray(v["CAindex"]).reshape(H.shape[4], 2))
    return out
