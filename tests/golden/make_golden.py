"""Generate tests/golden/projector_cases.npz: known-answer projector cases.

An independent transcription of the reference's loop structure
(forwardProjectACC.m:14-29, backwardProjectACC_new.m:14-26): for every
(aa, bb, cc) the lattice image tempspace(aa:Nnum:end, bb:Nnum:end) is
convolved with the (CAindex-cropped) PSF slice through
scipy.signal.convolve2d(..., mode='same'), which stands in for MATLAB's
conv2(..., 'same'); the back projection convolves with the slice rotated by
180 degrees and keeps the (aa, bb) lattice.  SciPy's 'same' centring equals
MATLAB's for odd kernel widths only, so every case here uses odd crops.

Run:  python tests/golden/make_golden.py     (writes projector_cases.npz)
"""
import os

import numpy as np
from scipy.signal import convolve2d

HERE = os.path.dirname(os.path.abspath(__file__))


def forward_loops(H, V, CAindex):
    M, _, N, _, Z = H.shape
    X, Y = V.shape[:2]
    out = np.zeros((X, Y))
    for aa in range(N):
        for bb in range(N):
            for cc in range(Z):
                lo, hi = CAindex[cc, 0] - 1, CAindex[cc, 1]
                Hs = H[lo:hi, lo:hi, aa, bb, cc].astype(np.float64)
                temp = np.zeros((X, Y))
                temp[aa::N, bb::N] = V[aa::N, bb::N, cc]
                out += convolve2d(temp, Hs, mode="same")
    return out


def backward_loops(H, I, CAindex):
    M, _, N, _, Z = H.shape
    X, Y = I.shape
    out = np.zeros((X, Y, Z))
    for cc in range(Z):
        for aa in range(N):
            for bb in range(N):
                lo, hi = CAindex[cc, 0] - 1, CAindex[cc, 1]
                filt = np.rot90(H[lo:hi, lo:hi, aa, bb, cc].astype(np.float64), 2)
                temp = convolve2d(I, filt, mode="same")
                out[aa::N, bb::N, cc] = temp[aa::N, bb::N]
    return out


def make_case(seed, M, N, Z, X, Y, crops=None):
    rng = np.random.default_rng(seed)
    H = rng.random((M, M, N, N, Z)).astype(np.float32)
    V = rng.random((X, Y, Z)).astype(np.float32)
    I = rng.random((X, Y)).astype(np.float32)
    if crops is None:
        ca = np.tile(np.array([[1, M]], dtype=np.int32), (Z, 1))
    else:
        ca = np.asarray(crops, dtype=np.int32)
    return dict(H=H, V=V, I=I, CAindex=ca, fwd=forward_loops(H, V, ca), adj=backward_loops(H, I, ca))


def main():
    cases = {
        # (seed, M, Nnum, Z, X, Y, crops)
        "small_full": (10, 9, 3, 2, 12, 12, None),
        "ragged": (11, 7, 3, 3, 13, 10, None),          # X, Y not multiples of Nnum
        "cropped": (12, 11, 3, 2, 15, 15, [[2, 10], [3, 9]]),  # odd per-depth crops
        "nnum5": (13, 15, 5, 2, 25, 20, None),
    }
    out = {}
    for name, (seed, M, N, Z, X, Y, crops) in cases.items():
        c = make_case(seed, M, N, Z, X, Y, crops)
        for k, v in c.items():
            out[f"{name}/{k}"] = v
    np.savez_compressed(os.path.join(HERE, "projector_cases.npz"), **out)
    print("wrote", sorted({k.split('/')[0] for k in out}))


if __name__ == "__main__":
    main()
