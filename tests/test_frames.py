"""Sensor-frame input: the TIFF reader, the ImageRect rectification and the
read_sensor_movie pipeline (ImageRect.m, read_sensor_movie.m)."""
import ctypes
import struct
import zlib

import numpy as np
import pytest

from tests.conftest import rel_l2


def write_tiff(path, img, compression=1, predictor=1, byteorder="<"):
    """Minimal baseline TIFF writer (one strip) for the reader tests."""
    img = np.ascontiguousarray(img)
    h, w = img.shape
    kind = {"u": 1, "i": 2, "f": 3}[img.dtype.kind]
    bits = img.dtype.itemsize * 8
    body = img.astype(img.dtype.newbyteorder(byteorder))
    if predictor == 2:
        d = body.astype(np.int64)
        d[:, 1:] = d[:, 1:] - d[:, :-1]
        body = d.astype(img.dtype).astype(img.dtype.newbyteorder(byteorder))
    raw = body.tobytes()
    if compression == 8:
        raw = zlib.compress(raw)
    entries = [(256, 3, 1, w), (257, 3, 1, h), (258, 3, 1, bits), (259, 3, 1, compression), (262, 3, 1, 1),
               (273, 4, 1, 0), (277, 3, 1, 1), (278, 3, 1, h), (279, 4, 1, len(raw)), (317, 3, 1, predictor),
               (339, 3, 1, kind)]
    ifd_off = 8
    data_off = ifd_off + 2 + 12 * len(entries) + 4
    out = bytearray((b"II" if byteorder == "<" else b"MM") + struct.pack(byteorder + "HI", 42, ifd_off))
    out += struct.pack(byteorder + "H", len(entries))
    for tag, typ, cnt, val in entries:
        if tag == 273:
            val = data_off
        packed = struct.pack(byteorder + ("H" if typ == 3 else "I"), val).ljust(4, b"\0")
        out += struct.pack(byteorder + "HHI", tag, typ, cnt) + packed
    out += struct.pack(byteorder + "I", 0)
    out += raw
    open(path, "wb").write(bytes(out))


@pytest.mark.parametrize("dtype", [np.uint16, np.uint8, np.float32, np.int32])
@pytest.mark.parametrize("comp,pred,bo", [(1, 1, "<"), (8, 1, "<"), (8, 2, "<"), (1, 1, ">")])
def test_tiff_roundtrip(tmp_path, dtype, comp, pred, bo):
    from sid_gb300 import read_tiff
    if pred == 2 and np.dtype(dtype).kind == "f":
        pytest.skip("horizontal differencing is defined for integer samples")
    rng = np.random.default_rng(1)
    img = (rng.uniform(0, 200, (37, 53))).astype(dtype)
    p = tmp_path / "f.tif"
    write_tiff(p, img, comp, pred, bo)
    np.testing.assert_array_equal(read_tiff(p), img)


@pytest.mark.parametrize("xc,yc,dx,M", [(100.3, 90.7, 15.2, 15), (57.0, 61.0, 15.0, 15), (99.5, 80.25, 11.7, 11)])
def test_oracle_image_rect_pinned(oracle, xc, yc, dx, M):
    """ImageRect.m:7-45 restated, against its definition: rectifying the images
    x and y themselves (bilinear interpolation reproduces them exactly) recovers
    the query grid, which steps dx/M, holds whole lenslets and puts the given
    centre on the middle pixel of its lenslet; the interpolation of a random
    image equals scipy's linear grid interpolator, NaN outside."""
    from scipy.interpolate import RegularGridInterpolator
    rows, cols = 181, 203
    xs = np.tile(np.arange(1.0, cols + 1), (rows, 1))
    ys = np.tile(np.arange(1.0, rows + 1)[:, None], (1, cols))
    gx = oracle.image_rect(xs, xc, yc, dx, M, crop=False)
    gy = oracle.image_rect(ys, xc, yc, dx, M, crop=False)
    xq = gx[np.isfinite(gx).any(axis=1)][0]
    yq = gy[:, np.isfinite(gy).any(axis=0)][:, 0]
    for q, c in ((xq, xc), (yq, yc)):
        assert q.size % M == 0
        f = q[np.isfinite(q)]
        np.testing.assert_allclose(np.diff(f), dx / M, rtol=1e-9)
        i = int(np.argmin(np.abs(np.nan_to_num(q, nan=-1e9) - (c + 1))))
        assert abs(q[i] - (c + 1)) < 1e-9 and i % M == M // 2
    img = np.random.default_rng(0).random((rows, cols))
    out = oracle.image_rect(img, xc, yc, dx, M, crop=False)
    fin = np.isfinite(yq)[:, None] & np.isfinite(xq)[None, :]
    assert np.array_equal(np.isfinite(out), fin)
    Yq, Xq = np.meshgrid(yq, xq, indexing="ij")
    ref = RegularGridInterpolator((np.arange(1.0, rows + 1), np.arange(1.0, cols + 1)), img)
    np.testing.assert_allclose(out[fin], ref(np.stack([Yq[fin], Xq[fin]], axis=1)), rtol=1e-12, atol=1e-12)


def test_rect_size_matches_oracle(sidlib, oracle):
    for rows, cols, xc, yc, dx, M, cuts in [(300, 310, 148.3, 151.7, 15.06, 15, (1, 2, 0, 1)),
                                            (200, 180, 90.0, 100.0, 14.8, 15, (0, 0, 0, 0)),
                                            (120, 130, 61.5, 58.25, 11.1, 11, (1, 0, 1, 0))]:
        ref = oracle.image_rect(np.zeros((rows, cols)), xc, yc, dx, M, True, cuts)
        c = np.asarray(cuts, dtype=np.int32)
        r_, c_ = ctypes.c_int64(), ctypes.c_int64()
        rc = sidlib.sid_image_rect_size(ctypes.c_int64(rows), ctypes.c_int64(cols), ctypes.c_double(xc),
                                        ctypes.c_double(yc), ctypes.c_double(dx), ctypes.c_int64(M), 1,
                                        c.ctypes.data_as(ctypes.c_void_p), ctypes.byref(r_), ctypes.byref(c_))
        assert rc == 0 and (r_.value, c_.value) == ref.shape and ref.shape[0] % M == 0


@pytest.mark.gpu
@pytest.mark.parametrize("u16", [True, False])
def test_rectify_frames_matches_oracle(gpu, oracle, u16):
    import sid_gb300 as s
    rng = np.random.default_rng(2)
    rows, cols, n = 300, 310, 4
    frames = rng.uniform(0, 4000, (rows, cols, n))
    frames = frames.astype(np.uint16) if u16 else frames.astype(np.float32)
    mask = (rng.uniform(0, 1, (rows, cols)) > 0.1).astype(np.float32) if u16 else None
    xc, yc, dx, M, cuts = 148.3, 151.7, 15.06, 15, (1, 2, 0, 1)
    mov, (R, C) = s.rectify_frames(frames, xc, yc, dx, M, True, cuts, mask)
    got = mov.cpu().numpy()
    for k in range(n):
        f = frames[:, :, k].astype(np.float64) * (mask if mask is not None else 1)
        ref = oracle.image_rect(f, xc, yc, dx, M, True, cuts)
        g = got[:, k].reshape(R, C, order="F")
        assert np.array_equal(np.isnan(g), np.isnan(ref))
        ok = ~np.isnan(ref)
        assert rel_l2(g[ok], ref[ok]) < 1e-6
    single = s.ImageRect(frames[:, :, 0].astype(np.float32), xc, yc, dx, M, True, *cuts).cpu().numpy()
    if not u16:
        np.testing.assert_array_equal(single, got[:, 0].reshape(R, C, order="F"))


@pytest.mark.gpu
def test_read_sensor_movie_pipeline(gpu, oracle, tmp_path):
    import sid_gb300 as s
    rng = np.random.default_rng(3)
    rows, cols = 200, 180
    imgs = [rng.uniform(0, 60000, (rows, cols)).astype(np.uint16) for _ in range(7)]
    for i, im in enumerate(imgs):
        write_tiff(tmp_path / f"frame_{i:03d}.tif", im, 8, 2)
    xc, yc, dx, N = 90.0, 100.0, 14.8, 15
    movie, size = s.read_sensor_movie(str(tmp_path), xc, yc, dx, N, True, {"start": 2, "step": 2, "end": 7},
                                      None, (0, 1, 1, 0), batch=2)
    got = movie.cpu().numpy()
    frames = [2, 4, 6]
    assert got.shape[1] == len(frames) and size[2] == 7
    for j, fidx in enumerate(frames):
        ref = oracle.image_rect(imgs[fidx - 1].astype(np.float64), xc, yc, dx, N, True, (0, 1, 1, 0))
        g = got[:, j].reshape(size[0], size[1], order="F")
        ok = ~np.isnan(ref)
        assert rel_l2(g[ok], ref[ok]) < 1e-6


@pytest.mark.gpu
def test_read_sensor_movie_frame_means(gpu, oracle, tmp_path):
    """frames.mean (read_sensor_movie.m:65-90): column j is the mean of the
    rectified frames list(j) .. list(j+1), both ends included."""
    import sid_gb300 as s
    rng = np.random.default_rng(4)
    rows, cols = 160, 150
    imgs = [rng.uniform(0, 60000, (rows, cols)).astype(np.uint16) for _ in range(8)]
    for i, im in enumerate(imgs):
        write_tiff(tmp_path / f"frame_{i:03d}.tif", im, 8, 2)
    xc, yc, dx, N = 75.0, 80.0, 14.8, 15
    movie, size = s.read_sensor_movie(str(tmp_path), xc, yc, dx, N, True, {"start": 1, "step": 3, "end": 8,
                                                                           "mean": 1})
    got = movie.cpu().numpy()
    starts = [1, 4, 7]
    assert got.shape[1] == len(starts) - 1
    for j in range(len(starts) - 1):
        refs = [oracle.image_rect(imgs[k - 1].astype(np.float64), xc, yc, dx, N, True, (0, 0, 0, 0))
                for k in range(starts[j], starts[j + 1] + 1)]
        ref = np.mean(refs, axis=0)
        g = got[:, j].reshape(size[0], size[1], order="F")
        ok = ~np.isnan(ref)
        assert rel_l2(g[ok], ref[ok]) < 1e-6
