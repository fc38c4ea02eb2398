"""Seeded synthetic inputs with the shapes of the SID benchmark configurations.

No public dataset is named for this path; these generators stand in for real
light-field recordings:

* PSF: every (aa, bb, cc) slice of H (M x M x Nnum x Nnum x Z) is a 2-D
  Gaussian with sigma growing linearly from 2 px at the central depth to 12 px
  at the outermost ones, centred at the PSF centre offset by the lenslet phase
  (aa - centre, bb - centre) px, normalised to sum 1.
* Volume: Gaussian blobs on a constant background.
* Library / movie: anisotropic neuron footprints, sparse exponential transients.

Arrays are returned Fortran-ordered (MATLAB layout) float32.
"""
from __future__ import annotations

import numpy as np

CONFIGS = {
    # Nnum, lenslets per side, depth planes, PSF side
    "cfg0": dict(Nnum=15, lenslets=15, Z=11, M=195),
    "cfg1": dict(Nnum=15, lenslets=67, Z=31, M=345),
}


def gaussian_psf(M: int, Nnum: int, Z: int, sigma_min=2.0, sigma_max=12.0, seed=0) -> np.ndarray:
    """H (M, M, Nnum, Nnum, Z) float32, Fortran order."""
    del seed  # deterministic construction; kept for a uniform signature
    ctr = M // 2
    cmid = (Z - 1) / 2.0
    pmid = (Nnum - 1) // 2
    i = np.arange(M, dtype=np.float64)
    H = np.empty((M, M, Nnum, Nnum, Z), dtype=np.float32, order="F")
    for c in range(Z):
        frac = abs(c - cmid) / cmid if cmid > 0 else 0.0
        sig = sigma_min + (sigma_max - sigma_min) * frac
        g = np.exp(-0.5 * ((i[None, :] - (ctr + np.arange(Nnum)[:, None] - pmid)) / sig) ** 2)  # (Nnum, M)
        g /= g.sum(axis=1, keepdims=True)
        # slice (aa, bb): outer product g[aa] (rows) x g[bb] (cols); sum = 1
        H[:, :, :, :, c] = np.einsum("ai,bj->ijab", g, g, optimize=True).astype(np.float32)
    return H


def blob_volume(X: int, Y: int, Z: int, n_blobs: int, sigma=(2.0, 2.0), amp="uniform", background=1e-3,
                seed=1) -> np.ndarray:
    """V (X, Y, Z) float32: Gaussian blobs (sigma in voxels) on a background."""
    rng = np.random.default_rng(seed)
    V = np.full((X, Y, Z), background, dtype=np.float64, order="F")
    cx = rng.uniform(0, X, n_blobs)
    cy = rng.uniform(0, Y, n_blobs)
    cz = rng.uniform(0, Z, n_blobs)
    sg = rng.uniform(sigma[0], sigma[1], n_blobs)
    if amp == "uniform":
        a = rng.uniform(0.5, 2.0, n_blobs)
    else:
        a = rng.lognormal(0.0, 0.5, n_blobs)
    for k in range(n_blobs):
        r = int(np.ceil(3 * sg[k]))
        x0, x1 = max(int(cx[k]) - r, 0), min(int(cx[k]) + r + 1, X)
        y0, y1 = max(int(cy[k]) - r, 0), min(int(cy[k]) + r + 1, Y)
        z0, z1 = max(int(cz[k]) - r, 0), min(int(cz[k]) + r + 1, Z)
        gx = np.exp(-0.5 * ((np.arange(x0, x1) - cx[k]) / sg[k]) ** 2)
        gy = np.exp(-0.5 * ((np.arange(y0, y1) - cy[k]) / sg[k]) ** 2)
        gz = np.exp(-0.5 * ((np.arange(z0, z1) - cz[k]) / sg[k]) ** 2)
        V[x0:x1, y0:y1, z0:z1] += a[k] * gx[:, None, None] * gy[None, :, None] * gz[None, None, :]
    return np.asfortranarray(V.astype(np.float32))


def config_inputs(name: str, seed_psf=0, seed_vol=1):
    """(H, V) for cfg0 (40 blobs, sigma 2, U(0.5,2) amplitudes) or cfg1 (2000
    blobs, sigma U(2,4), log-normal amplitudes)."""
    c = CONFIGS[name]
    X = c["Nnum"] * c["lenslets"]
    H = gaussian_psf(c["M"], c["Nnum"], c["Z"], seed=seed_psf)
    if name == "cfg0":
        V = blob_volume(X, X, c["Z"], 40, sigma=(2.0, 2.0), amp="uniform", seed=seed_vol)
    else:
        V = blob_volume(X, X, c["Z"], 2000, sigma=(2.0, 4.0), amp="lognormal", seed=seed_vol)
    return H, V


def poisson_image(I: np.ndarray, scale=1000.0, seed=2) -> np.ndarray:
    """Poisson-noised sensor image (counts / scale)."""
    rng = np.random.default_rng(seed)
    return np.asfortranarray((rng.poisson(np.maximum(I, 0) * scale) / scale).astype(np.float32))
