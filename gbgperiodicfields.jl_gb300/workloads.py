"""Seeded synthetic inputs with the shapes and value distributions of the benchmark
configurations (no public dataset is involved):

  fields  real, periodic on [0, 2pi)^3, random Fourier modes with |k| <= kmax, amplitude
          proportional to |k|^(-11/6) and uniform phases; vector fields divergence-
          projected (u_hat -= k (k . u_hat) / |k|^2); the velocity-gradient tensor
          computed spectrally (i k_j u_hat_i); every component scaled to unit RMS.
  points  uniform in the box, or 70% uniform + 30% in Gaussian blobs (sigma = 0.05),
          wrapped into the box.

Mode coefficients are drawn on the host with numpy's PCG64 so that every device (and the
host) builds the same field; the inverse FFT runs on the requested torch device.
All returned arrays are column-major (Fortran order), like the reference's.
"""
from __future__ import annotations

import numpy as np
import torch

TWO_PI = 2 * np.pi


def _mode_coefficients(kmax: int, ncomp: int, seed: int):
    rng = np.random.Generator(np.random.PCG64(seed))
    ks = np.arange(-kmax, kmax + 1)
    KX, KY, KZ = np.meshgrid(ks, ks, np.arange(0, kmax + 1), indexing="ij")
    kk = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    mask = (kk > 0) & (kk <= kmax)
    amp = np.zeros_like(kk)
    amp[mask] = kk[mask] ** (-11.0 / 6.0)
    phases = rng.random((ncomp,) + kk.shape)
    mags = rng.standard_normal((ncomp,) + kk.shape)
    coef = amp[None] * mags * np.exp(2j * np.pi * phases)
    return KX, KY, KZ, coef


def spectral_field(n, ncomp: int = 1, kmax: int = 8, seed: int = 0, project: bool = False,
                   gradient: bool = False, device="cpu", dtype=torch.float64):
    """An (Nx, Ny, Nz, C) column-major field; C = ncomp, or ncomp + 3*ncomp with gradient.
    Returns a numpy array for device == 'cpu', else a torch tensor on that device."""
    nx, ny, nz = (int(v) for v in n)
    kmax = min(kmax, nx // 2 - 1, ny // 2 - 1, nz // 2 - 1)
    KX, KY, KZ, coef = _mode_coefficients(kmax, ncomp, seed)
    if project and ncomp == 3:
        k2 = (KX ** 2 + KY ** 2 + KZ ** 2).astype(np.float64)
        k2[k2 == 0] = 1.0
        kdotu = KX * coef[0] + KY * coef[1] + KZ * coef[2]
        coef = coef - np.stack([KX, KY, KZ]) * (kdotu / k2)[None]
    comps = [coef[c] for c in range(ncomp)]
    if gradient:
        # d u_i / d x_j = i k_j u_i ; stored column-major as (i, j) -> fibre i + 3 j
        for j, K in enumerate((KX, KY, KZ)):
            for i in range(ncomp):
                comps.append(1j * K * coef[i])
    dev = torch.device(device)
    cdtype = torch.complex128 if dtype == torch.float64 else torch.complex64
    out = torch.empty((len(comps), nz, ny, nx), dtype=dtype, device=dev)
    ix = np.mod(KX, nx)
    iy = np.mod(KY, ny)
    iz = KZ
    for c, cf in enumerate(comps):
        spec = torch.zeros((nx, ny, nz // 2 + 1), dtype=cdtype, device=dev)
        spec[torch.from_numpy(ix.ravel()).to(dev), torch.from_numpy(iy.ravel()).to(dev),
             torch.from_numpy(iz.ravel()).to(dev)] = torch.from_numpy(cf.ravel()).to(dev, cdtype)
        real = torch.fft.irfftn(spec, s=(nx, ny, nz), dim=(0, 1, 2))
        real = real / real.square().mean().sqrt().clamp_min(1e-300)
        out[c] = real.permute(2, 1, 0)
        del spec, real
    field = out.permute(3, 2, 1, 0)  # (Nx, Ny, Nz, C) column-major
    if dev.type == "cpu":
        return np.asfortranarray(field.numpy())
    return field


def uniform_points(m: int, seed: int = 0, length: float = TWO_PI, dtype=np.float64):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.asfortranarray((length * rng.random((m, 3))).astype(dtype))


def clustered_points(m: int, seed: int = 0, length: float = TWO_PI, cluster_fraction: float = 0.3,
                     nblobs: int = 1000, sigma: float = 0.05, dtype=np.float64):
    """70% uniform plus 30% in nblobs Gaussian blobs of width sigma, wrapped."""
    rng = np.random.Generator(np.random.PCG64(seed))
    mc = int(round(cluster_fraction * m))
    mu = m - mc
    uni = length * rng.random((mu, 3))
    centres = length * rng.random((nblobs, 3))
    which = rng.integers(0, nblobs, mc)
    blob = centres[which] + sigma * rng.standard_normal((mc, 3))
    pts = np.concatenate([uni, np.mod(blob, length)], axis=0)
    pts = pts[rng.permutation(m)]
    return np.asfortranarray(pts.astype(dtype))
