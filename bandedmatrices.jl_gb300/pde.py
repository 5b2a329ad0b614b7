"""Band storage of the 5-point variable-coefficient diffusion operator
-div(k grad u) on a G x G grid (or an H x G strip; unit spacing, zero Dirichlet
boundary), natural (row-major) ordering: n = G^2 (H G), bandwidths (G, G).  This is
the operator of the differentiated PDE solve (the reference's examples/finitedifference_2d.jl builds the
constant-coefficient case with BandedMatrices); face coefficients are harmonic means
of the cell values of k, so A is symmetric positive definite.
"""
from __future__ import annotations

import numpy as np
import torch

from .banded import BandedMatrix, band_storage


def gaussian_field(G: int, corr: float, seed: int) -> np.ndarray:
    """Seeded Gaussian random field on a G x G grid with correlation length `corr` cells
    (white noise filtered by a Gaussian kernel in Fourier space), unit variance."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((G, G))
    k = np.fft.fftfreq(G)
    kx, ky = np.meshgrid(k, k, indexing="ij")
    filt = np.exp(-0.5 * (2 * np.pi * corr) ** 2 * (kx ** 2 + ky ** 2))
    g = np.real(np.fft.ifft2(np.fft.fft2(w) * filt))
    return (g - g.mean()) / g.std()


def diffusion_band_data(kcell: np.ndarray) -> np.ndarray:
    """(2G+1) x n band storage (bandwidths (G, G)) of the operator for cell coefficients
    kcell on an H x G grid (H rows, G columns; n = H G, natural ordering p = j + G i)."""
    H, G = kcell.shape
    n = H * G
    hm = lambda a, b: 2.0 * a * b / (a + b)
    kx = np.zeros((H + 1, G))  # faces between (i-1, j) and (i, j), i = 0..H
    kx[1:H] = hm(kcell[:-1], kcell[1:])
    kx[0], kx[H] = kcell[0], kcell[-1]
    ky = np.zeros((H, G + 1))
    ky[:, 1:G] = hm(kcell[:, :-1], kcell[:, 1:])
    ky[:, 0], ky[:, G] = kcell[:, 0], kcell[:, -1]
    # index p = j + G*i  (i: row of the grid, j: column) -> neighbours p+-1 (j+-1), p+-G (i+-1)
    data = np.zeros((2 * G + 1, n))
    u = G
    diag = (kx[:-1] + kx[1:] + ky[:, :-1] + ky[:, 1:]).reshape(-1)
    data[u, :] = diag
    # A[p, p+1] = -ky[i, j+1] for j < G-1: storage row u + p - (p+1) = u - 1, column p+1
    east = -ky[:, 1:G]                       # (H, G-1): face between (i,j) and (i,j+1)
    for i in range(H):
        p = i * G + np.arange(G - 1)
        data[u - 1, p + 1] = east[i]        # A[p, p+1]
        data[u + 1, p] = east[i]            # A[p+1, p]
    south = -kx[1:H]                        # (H-1, G): face between (i,j) and (i+1,j)
    for i in range(H - 1):
        p = i * G + np.arange(G)
        data[u - G, p + G] = south[i]       # A[p, p+G]
        data[u + G, p] = south[i]           # A[p+G, p]
    return data


def diffusion_band(kcell: np.ndarray, dtype=torch.float64, device="cuda") -> BandedMatrix:
    """The operator for cell coefficients kcell (H x G, usually G x G) as a device
    BandedMatrix with bandwidths (G, G)."""
    G = kcell.shape[1]
    data = diffusion_band_data(kcell)
    d = band_storage(2 * G + 1, data.shape[1], dtype, device)
    d.copy_(torch.from_numpy(data))
    return BandedMatrix(d, data.shape[1], G, G)
