"""The tensor-core GEMM's tile planner (host code, no GPU needed): the tile
width and K split that sid_gram / sid_cross and the solvers' contractions use,
against a restatement of its cost model:

  waves x (K blocks per CTA x BN / efficiency(BN) + 1024) + s m n / 4096 (s > 1)

with waves = ceil(tiles x s / SMs), efficiencies 1.0 / 0.78 / 0.55 / 0.45 for
BN = 256 / 192 / 128 / 64 (measured on GB300), and only the tiles on and above
the diagonal for a symmetric product."""
import ctypes

import numpy as np
import pytest


def _cdiv(a, b):
    return -(-a // b)


def _tiles(m, n, bn, sym):
    tm, tn = _cdiv(m, 128), _cdiv(n, bn)
    if not sym:
        return tm * tn
    return sum(min(tm, _cdiv(j * bn + bn, 128)) for j in range(tn))


def _model(m, n, k, sym, sms):
    nkb = _cdiv(k, 64)
    best, pick = None, None
    for bn, eff in zip((256, 192, 128, 64), (1.0, 0.78, 0.55, 0.45)):
        t_ = _tiles(m, n, bn, sym)
        for s0 in range(1, 65):
            if s0 > 1 and nkb // s0 < 8:
                break
            kb = _cdiv(nkb, s0)
            s = _cdiv(nkb, kb)
            w = _cdiv(t_ * s, sms)
            t = w * (kb * bn / eff + 1024.0) + (s * m * n / 4096.0 if s > 1 else 0.0)
            if best is None or t < best * (1 - 1e-9):
                best, pick = t, (bn, s)
    return pick


def _plan(lib, m, n, k, sym, sms=152):
    bn, sk = ctypes.c_int(), ctypes.c_int()
    rc = lib.sid_gemm_tile_plan(ctypes.c_int64(m), ctypes.c_int64(n), ctypes.c_int64(k), int(sym), sms,
                                ctypes.byref(bn), ctypes.byref(sk))
    assert rc == 0
    return bn.value, sk.value


P = 1010025


@pytest.mark.parametrize("m,n,k,sym,expect", [
    (800, 800, P, True, (256, 8)),      # Gram S'S of the temporal NNLS: one full wave of 19 x 8 CTAs
    (800, 3000, P, False, (256, 9)),    # cross product S'Y: 84 tiles x 9 splits, five waves
    (800, 3000, 800, False, (192, 1)),  # G d of an NNLS iteration: one wave of 112 CTAs
    (1500, 5000, P, False, None),
    (P, 800, 3000, False, None),        # S_update's pixel-by-rank product
    (300, 300, 200000, True, None),
])
def test_tile_plan_follows_the_model(sidlib, m, n, k, sym, expect):
    from sid_gb300 import _lib
    lib = _lib.load()
    got = _plan(lib, m, n, k, sym)
    assert got == _model(m, n, k, sym, 152)
    if expect is not None:
        assert got == expect


def test_tile_plan_limits(sidlib):
    """Splits keep at least 8 K blocks each (K = 600: no split), and the plan
    follows the SM count."""
    from sid_gb300 import _lib
    lib = _lib.load()
    assert _plan(lib, 512, 512, 600, False)[1] == 1
    rng = np.random.default_rng(0)
    for _ in range(40):
        m, n = int(rng.integers(64, 4000)), int(rng.integers(64, 4000))
        k = int(rng.integers(64, 2_000_000))
        sms = int(rng.choice([132, 148, 152, 160]))
        sym = bool(rng.random() < 0.3)
        if sym:
            n = m
        assert _plan(lib, m, n, k, sym, sms) == _model(m, n, k, sym, sms), (m, n, k, sym, sms)
