"""The runs the weakly observed voxels are recomputed in (host code, no GPU):
every listed voxel lies in exactly one run, runs are straight and at most 24
long, a maximal line is split into near-equal pieces, and the runs come plane
by plane (the depth ranges of the back projection index them that way)."""
import ctypes

import numpy as np
import pytest


def _plan(lib, vox, N, Lx, Ly):
    lst = np.ascontiguousarray(np.asarray(sorted(vox), dtype=np.int32))
    nc, nr = ctypes.c_int64(), ctypes.c_int64()
    assert lib.sid_weak_runs_plan(lst.ctypes.data, len(lst), N, Lx, Ly, None, 0, ctypes.byref(nc),
                                  ctypes.byref(nr)) == 0
    runs = np.zeros((nc.value + nr.value, 4), dtype=np.int32)
    assert lib.sid_weak_runs_plan(lst.ctypes.data, len(lst), N, Lx, Ly, runs.ctypes.data, len(runs), ctypes.byref(nc),
                                  ctypes.byref(nr)) == 0
    return runs, nc.value


def _border_set(rng, N, Z, Lx, Ly, planes):
    plane = Lx * Ly
    vox = set()
    for pl in planes:
        for _ in range(int(rng.integers(1, 4))):
            side = int(rng.integers(0, 4))
            a, b = sorted(rng.integers(0, (Ly if side < 2 else Lx), 2))
            for t in range(a, b + 1):
                u, v = {0: (0, t), 1: (Lx - 1, t), 2: (t, 0), 3: (t, Ly - 1)}[side]
                vox.add(pl * plane + v * Lx + u)
        for _ in range(int(rng.integers(0, 6))):  # isolated voxels anywhere in the plane
            vox.add(pl * plane + int(rng.integers(0, Ly)) * Lx + int(rng.integers(0, Lx)))
    return vox


@pytest.mark.parametrize("seed", range(6))
def test_runs_cover_the_voxels(sidlib, seed):
    from sid_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(seed)
    N, Z, Lx, Ly = 5, 7, 67, 61
    planes = sorted(rng.choice(N * N * Z, 20, replace=False))
    vox = _border_set(rng, N, Z, Lx, Ly, planes)
    runs, nc = _plan(lib, vox, N, Lx, Ly)
    plane = Lx * Ly
    seen = []
    for k, (pl, fixed, start, ln) in enumerate(runs):
        assert 1 <= ln <= 24
        col = k < nc
        for j in range(ln):
            u, v = (fixed, start + j) if col else (start + j, fixed)
            assert 0 <= u < Lx and 0 <= v < Ly
            seen.append(pl * plane + v * Lx + u)
    assert sorted(seen) == sorted(vox)  # each voxel exactly once
    # plane by plane within the column runs and within the row runs
    assert np.all(np.diff(runs[:nc, 0]) >= 0) and np.all(np.diff(runs[nc:, 0]) >= 0)


def test_long_line_splits_evenly(sidlib):
    """A full border column of 61 voxels: three runs of 20-21."""
    from sid_gb300 import _lib
    lib = _lib.load()
    Lx, Ly = 67, 61
    vox = {3 * Lx * Ly + v * Lx for v in range(Ly)}
    runs, nc = _plan(lib, vox, 5, Lx, Ly)
    assert nc == 3 and len(runs) == 3
    assert sorted(runs[:, 3].tolist()) == [20, 20, 21]
    assert runs[:, 2].tolist() == [0, 20, 40] or sorted(runs[:, 2].tolist()) == [0, 21, 41]


def test_runs_reject_unsorted(sidlib):
    from sid_gb300 import _lib
    lib = _lib.load()
    lst = np.array([5, 3], dtype=np.int32)
    nc, nr = ctypes.c_int64(), ctypes.c_int64()
    assert lib.sid_weak_runs_plan(lst.ctypes.data, 2, 5, 10, 10, None, 0, ctypes.byref(nc), ctypes.byref(nr)) != 0
