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
    "225x225x11": dict(Nnum=15, lenslets=15, Z=11, M=195),
    "1005x1005x31": dict(Nnum=15, lenslets=67, Z=31, M=345),
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
    """(H, V) for the 225 x 225 x 11 frame (40 blobs, sigma 2, U(0.5,2)
    amplitudes) or the 1005 x 1005 x 31 frame (2000 blobs, sigma U(2,4),
    log-normal amplitudes)."""
    c = CONFIGS[name]
    X = c["Nnum"] * c["lenslets"]
    H = gaussian_psf(c["M"], c["Nnum"], c["Z"], seed=seed_psf)
    if name == "225x225x11":
        V = blob_volume(X, X, c["Z"], 40, sigma=(2.0, 2.0), amp="uniform", seed=seed_vol)
    else:
        V = blob_volume(X, X, c["Z"], 2000, sigma=(2.0, 4.0), amp="lognormal", seed=seed_vol)
    return H, V


def poisson_image(I: np.ndarray, scale=1000.0, seed=2) -> np.ndarray:
    """Poisson-noised sensor image (counts / scale)."""
    rng = np.random.default_rng(seed)
    return np.asfortranarray((rng.poisson(np.maximum(I, 0) * scale) / scale).astype(np.float32))


def neuron_volume(X: int, Y: int, Z: int, K: int, seed=5):
    """K anisotropic Gaussian neuron footprints (sigma_xy U(2,4), sigma_z U(1,2)
    voxels, boxes of +-3 sigma) at uniform positions in an X x Y x Z volume,
    summed into one float32 volume.  Returns (volume, centers (K x 3, 1-based
    MATLAB coordinates))."""
    rng = np.random.default_rng(seed)
    cx, cy, cz = rng.uniform(1, X, K), rng.uniform(1, Y, K), rng.uniform(1, Z, K)
    sxy, sz = rng.uniform(2, 4, K), rng.uniform(1, 2, K)
    vol = np.zeros((X, Y, Z), dtype=np.float32, order="F")
    for k in range(K):
        r, rz = int(np.ceil(3 * sxy[k])), int(np.ceil(3 * sz[k]))
        x0, x1 = max(int(cx[k]) - 1 - r, 0), min(int(cx[k]) + r, X)
        y0, y1 = max(int(cy[k]) - 1 - r, 0), min(int(cy[k]) + r, Y)
        z0, z1 = max(int(cz[k]) - 1 - rz, 0), min(int(cz[k]) + rz, Z)
        gx = np.exp(-0.5 * ((np.arange(x0, x1) + 1 - cx[k]) / sxy[k]) ** 2)
        gy = np.exp(-0.5 * ((np.arange(y0, y1) + 1 - cy[k]) / sxy[k]) ** 2)
        gz = np.exp(-0.5 * ((np.arange(z0, z1) + 1 - cz[k]) / sz[k]) ** 2)
        vol[x0:x1, y0:y1, z0:z1] += (gx[:, None, None] * gy[None, :, None] * gz[None, None, :]).astype(np.float32)
    return vol, np.stack([cx, cy, cz], 1)


def transient_movie(A, F: int, seed=7, event_rate=0.025, tau_frames=6.0, snr=10.0):
    """Temporal NNLS inputs on the GPU from a library A (P x K, CUDA float32,
    column-major): T_true (K x F) of sparse exponential transients (events with
    probability `event_rate` per frame -- 0.5 Hz at 20 Hz --, amplitudes
    U(0.5, 1.5), decay tau_frames = 0.3 s), and the movie Y = A T_true + b + noise
    with a constant background b = rms/snr and Gaussian noise of deviation
    rms/snr.  Returns (Y16 half, Yf float32, T_true), Y column-major P x F."""
    import torch
    K = A.shape[1]
    g = torch.Generator(device=A.device).manual_seed(seed)
    ev = (torch.rand(K, F, generator=g, device=A.device) < event_rate).float() * \
        (0.5 + torch.rand(K, F, generator=g, device=A.device))
    kern = torch.exp(-torch.arange(0, 40, device=A.device, dtype=torch.float32) / tau_frames)
    T = torch.nn.functional.conv1d(ev[:, None, :], kern.flip(0)[None, None, :], padding=39)[:, 0, :F]
    sig = A.T.contiguous().T @ T
    rms = sig.pow(2).mean().sqrt()
    Yf = sig + rms / snr + rms / snr * torch.randn(sig.shape, generator=g, device=A.device)
    del sig
    Y16 = Yf.half().T.contiguous().T
    Yf = Yf.T.contiguous().T
    return Y16, Yf, T
