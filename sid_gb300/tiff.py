"""Baseline TIFF reader for sensor frames (the imread(..., 'tiff') of
read_sensor_movie.m:88-97): the first image of a little- or big-endian file,
grey-scale, strips, uncompressed or deflate (with or without horizontal
differencing), 8/16/32-bit unsigned or signed integers or 32/64-bit floats.
Tiled and other compressed layouts raise.  Returns a (rows, cols) array."""
from __future__ import annotations

import struct
import zlib

import numpy as np

_TYPES = {1: "B", 2: "s", 3: "H", 4: "I", 5: "II", 6: "b", 7: "B", 8: "h", 9: "i", 10: "ii", 11: "f", 12: "d",
          16: "Q"}


def read_tiff(path) -> np.ndarray:
    with open(path, "rb") as f:
        data = f.read()
    bo = {b"II": "<", b"MM": ">"}.get(data[:2])
    if bo is None:
        raise ValueError(f"{path}: not a TIFF file")
    magic, ifd = struct.unpack(bo + "HI", data[2:8])
    if magic != 42:
        raise ValueError(f"{path}: BigTIFF or unknown variant ({magic})")
    (n,) = struct.unpack(bo + "H", data[ifd:ifd + 2])
    tags = {}
    for e in range(n):
        tag, typ, cnt, val = struct.unpack(bo + "HHI4s", data[ifd + 2 + 12 * e:ifd + 14 + 12 * e])
        fmt = _TYPES.get(typ)
        if fmt is None:
            continue
        size = struct.calcsize(bo + fmt) * cnt
        raw = val if size <= 4 else data[struct.unpack(bo + "I", val)[0]:][:size]
        tags[tag] = struct.unpack(bo + fmt * cnt, raw[:size])
    width, height = tags[256][0], tags[257][0]
    bits = tags.get(258, (1,))[0]
    comp = tags.get(259, (1,))[0]
    spp = tags.get(277, (1,))[0]
    fmt_code = tags.get(339, (1,))[0]
    pred = tags.get(317, (1,))[0]
    if 322 in tags:
        raise ValueError(f"{path}: tiled TIFF is not supported")
    if spp != 1:
        raise ValueError(f"{path}: {spp} samples per pixel (grey-scale frames expected)")
    kind = {1: "u", 2: "i", 3: "f"}[fmt_code]
    dtype = np.dtype(bo + kind + str(bits // 8))
    offs, counts = tags[273], tags[279]
    chunks = []
    for o, c in zip(offs, counts):
        blob = data[o:o + c]
        if comp in (8, 32946):
            blob = zlib.decompress(blob)
        elif comp != 1:
            raise ValueError(f"{path}: compression {comp} is not supported")
        chunks.append(blob)
    img = np.frombuffer(b"".join(chunks), dtype=dtype)[: width * height].reshape(height, width)
    if pred == 2:
        img = np.cumsum(img, axis=1, dtype=dtype)
    return img.astype(dtype.newbyteorder("="))
