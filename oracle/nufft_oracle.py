"""CPU restatement of the reference's spectral transfers (test infrastructure only).

Only the tests use this module, as the checker of the device NUFFT path; nothing in the
package imports it.  numpy throughout, sized for the small grids the tests use.

Restated from GBGPeriodicFields.jl src/Interpolation.jl:
  DirectDFT                 1386-1404 (the definition), 1440-1466 (_dft_axis)
      f(x_p)      = (1/N) sum_stored alpha(k) Re(f_hat(k) exp(i k.(x_p - o)))
      (W^T q)(k)  = sum_p q_p exp(-i k.(x_p - o))        at every stored k
  _stencil_half             1634-1635
  _es_weights               1638-1645
  _es_window_transform      1652-1662
  _nufft_width/_nufft_beta  1670-1677
  _nufft_deconvolution      1682-1712
  NUFFT type 2 / type 1     1984-2062 (_nufft_gather_kernel! 1864-1914, _nufft_spread_kernel! 1919-1950)
  inner of spectral fields  src/Reductions.jl:856-883 (Parseval: Re sum alpha f conj(g) / N^2)

Conventions: a grid is a dict {"n": (3,), "domain": (3,), "origin": (3,)}; fields are
column-major numpy arrays (x fastest), spectral fields the stored rfft half-spectrum with
the half axis `half` (0-based), fibres trailing; positions (M, 3); values (M, ncomp).
"""
from __future__ import annotations

import math

import numpy as np


def grid(n, domain=(2 * np.pi,) * 3, origin=(0.0, 0.0, 0.0)):
    return {"n": tuple(int(v) for v in n), "domain": tuple(float(v) for v in domain),
            "origin": tuple(float(v) for v in origin)}


def stored_shape(n, half):
    return tuple(v // 2 + 1 if d == half else v for d, v in enumerate(n))


def _fft_axes(half):
    return tuple(d for d in range(3) if d != half) + (half,)


def to_spectral(phys, half):
    """Unnormalized forward real FFT (the reference's to_spectral)."""
    return np.fft.rfftn(phys, axes=_fft_axes(half))


def to_physical(spec, n, half):
    axes = _fft_axes(half)
    return np.fft.irfftn(spec, s=tuple(n[d] for d in axes), axes=axes)


# ------------------------------------------------------------------ DirectDFT


def dft_axis(stored, n, domain, is_half, dtype=np.float64):
    """_dft_axis: true wavenumbers and the half-axis Parseval weights."""
    unit = dtype(2) * dtype(np.pi) / dtype(domain)
    k = np.empty(stored, dtype=dtype)
    for i in range(stored):
        f = i if (is_half or i < (n + 1) // 2) else i - n
        k[i] = unit * dtype(f)
    if is_half:
        w = np.full(stored, 2.0, dtype=dtype)
        w[0] = 1.0
        if n % 2 == 0:
            w[-1] = 1.0
    else:
        w = np.ones(stored, dtype=dtype)
    return k, w


def _axes(g, half):
    sh = stored_shape(g["n"], half)
    return [dft_axis(sh[d], g["n"][d], g["domain"][d], d == half) for d in range(3)]


def direct_interpolate(fh, g, half, positions):
    """DirectDFT interpolate: (M, ncomp) real."""
    axes = _axes(g, half)
    fh = np.asarray(fh)
    ncomp = int(np.prod(fh.shape[3:])) if fh.ndim > 3 else 1
    F = fh.reshape(fh.shape[:3] + (ncomp,), order="F")
    alpha = axes[0][1][:, None, None] * axes[1][1][None, :, None] * axes[2][1][None, None, :]
    N = float(np.prod(g["n"]))
    out = np.empty((positions.shape[0], ncomp))
    for p in range(positions.shape[0]):
        e = [np.exp(1j * axes[d][0] * (positions[p, d] - g["origin"][d])) for d in range(3)]
        phase = e[0][:, None, None] * e[1][None, :, None] * e[2][None, None, :]
        for c in range(ncomp):
            out[p, c] = np.sum(alpha * np.real(F[..., c] * phase)) / N
    return out


def direct_anterpolate(g, half, positions, q):
    """DirectDFT anterpolate: (W^T q)(k) at every stored k, (stored..., ncomp) complex."""
    axes = _axes(g, half)
    q = np.asarray(q).reshape(positions.shape[0], -1, order="F")
    sh = stored_shape(g["n"], half)
    out = np.zeros(sh + (q.shape[1],), dtype=np.complex128)
    for p in range(positions.shape[0]):
        e = [np.exp(-1j * axes[d][0] * (positions[p, d] - g["origin"][d])) for d in range(3)]
        phase = e[0][:, None, None] * e[1][None, :, None] * e[2][None, None, :]
        for c in range(q.shape[1]):
            out[..., c] += q[p, c] * phase
    return out


def inner_spectral(fh, gh, n, half):
    """Re sum alpha f conj(g) / N^2 over the stored modes (every fibre)."""
    sh = stored_shape(n, half)
    _, w = dft_axis(sh[half], n[half], 1.0, True)
    shape = [1, 1, 1]
    shape[half] = sh[half]
    alpha = w.reshape(shape)
    F = np.asarray(fh).reshape(sh + (-1,), order="F")
    G = np.asarray(gh).reshape(sh + (-1,), order="F")
    return float(np.sum(alpha[..., None] * np.real(F * np.conj(G)))) / float(np.prod(n)) ** 2


# ----------------------------------------------------------------- the window


def nufft_width(tolerance):
    return max(4, math.ceil(-math.log10(tolerance)) + 2)


def nufft_beta(width, dtype=np.float64):
    return dtype(dtype(23) / dtype(10) * dtype(width))


def stencil_half(t, W):
    return (W + 1) // 2 if (W % 2 == 1 and t < 0.5) else W // 2


def es_weights(t, beta, W, dtype=np.float64):
    half = stencil_half(t, W)
    w = np.empty(W, dtype=dtype)
    for i in range(1, W + 1):
        z = dtype(dtype(2) * (dtype(t) - dtype(i - half))) / dtype(W)
        r = dtype(1) - z * z
        w[i - 1] = np.exp(dtype(beta) * (np.sqrt(max(r, dtype(0))) - dtype(1)))
    return w, half


def locate(x, o, d, dtype=np.float64):
    ci = (dtype(x) - dtype(o)) / dtype(d)
    base = math.floor(ci)
    return base, dtype(ci - dtype(base))


def es_window_transform(omega, beta, width, dtype=np.float64, quadrature_points=256):
    half_width = dtype(width) / dtype(2)
    pi = dtype(np.pi)
    acc = dtype(0)
    for q in range(quadrature_points + 1):
        theta = -pi / dtype(2) + pi * dtype(q) / dtype(quadrature_points)
        trap = dtype(0.5) if q in (0, quadrature_points) else dtype(1)
        acc += trap * np.exp(dtype(beta) * (np.cos(theta) - dtype(1))) * np.cos(omega * half_width * np.sin(theta)) * np.cos(theta)
    return half_width * (pi / dtype(quadrature_points)) * acc


def deconvolution_axis(n, is_half, sigma, width, beta, dtype=np.float64):
    stored = n // 2 + 1 if is_half else n
    out = np.empty(stored, dtype=dtype)
    for i in range(stored):
        f = i if (is_half or i < (n + 1) // 2) else i - n
        omega = dtype(2) * dtype(np.pi) * dtype(f) / dtype(sigma * n)
        out[i] = dtype(1) / es_window_transform(omega, beta, width, dtype)
    if n % 2 == 0:
        out[stored - 1 if is_half else n // 2] = 0
    return out


def deconvolution(n, half, sigma, width, beta, dtype=np.float64):
    a = [deconvolution_axis(n[d], d == half, sigma, width, beta, dtype) for d in range(3)]
    return a[0][:, None, None] * a[1][None, :, None] * a[2][None, None, :]


def _fine_grid(g, sigma):
    n = tuple(sigma * v for v in g["n"])
    return {"n": n, "domain": g["domain"], "origin": g["origin"],
            "spacing": tuple(g["domain"][d] / n[d] for d in range(3))}


def window_gather(fg, field, positions, W, beta, dtype=np.float64):
    """_nufft_gather_kernel!: (M, ncomp), accumulated in the reference's loop order."""
    n = fg["n"]
    F = np.asarray(field).reshape(n + (-1,), order="F")
    out = np.empty((positions.shape[0], F.shape[3]), dtype=dtype)
    for p in range(positions.shape[0]):
        ws, idx = [], []
        for d in range(3):
            base, t = locate(positions[p, d], fg["origin"][d], dtype(fg["spacing"][d]), dtype)
            w, half = es_weights(t, beta, W, dtype)
            ws.append(w)
            idx.append(np.array([(base + (i - half)) % n[d] for i in range(1, W + 1)]))
        sub = F[np.ix_(idx[0], idx[1], idx[2])]
        wt = (ws[1][None, :, None] * ws[2][None, None, :]) * ws[0][:, None, None]
        out[p] = np.einsum("ijk,ijkc->c", wt, sub)
    return out


def window_spread(fg, positions, q, W, beta, dtype=np.float64):
    """_nufft_spread_kernel!: the oversampled field (n..., ncomp), sums in point order."""
    n = fg["n"]
    q = np.asarray(q).reshape(positions.shape[0], -1, order="F")
    F = np.zeros(n + (q.shape[1],), dtype=dtype)
    for p in range(positions.shape[0]):
        ws, idx = [], []
        for d in range(3):
            base, t = locate(positions[p, d], fg["origin"][d], dtype(fg["spacing"][d]), dtype)
            w, half = es_weights(t, beta, W, dtype)
            ws.append(w)
            idx.append(np.array([(base + (i - half)) % n[d] for i in range(1, W + 1)]))
        wt = (ws[1][None, :, None] * ws[2][None, None, :]) * ws[0][:, None, None]
        for c in range(q.shape[1]):
            np.add.at(F[..., c], np.ix_(idx[0], idx[1], idx[2]), wt * q[p, c])
    return F


def shared_slices(n, nf, is_half):
    if is_half:
        k = (n + 1) // 2
        return [(slice(0, k), slice(0, k))]
    pos, neg = (n + 1) // 2, n - n // 2 - 1
    pairs = [(slice(0, pos), slice(0, pos))]
    if neg > 0:
        pairs.append((slice(n - neg, n), slice(nf - neg, nf)))
    return pairs


def nufft_interpolate(fh, g, half, positions, W, beta, sigma=2, dtype=np.float64):
    """NUFFT type 2 (interpolate! with a NUFFT)."""
    fg = _fine_grid(g, sigma)
    ratio = float(np.prod(fg["n"]) / np.prod(g["n"]))
    D = deconvolution(g["n"], half, sigma, W, beta, dtype)
    fh = np.asarray(fh)
    ncomp = int(np.prod(fh.shape[3:])) if fh.ndim > 3 else 1
    F = fh.reshape(fh.shape[:3] + (ncomp,), order="F") * D[..., None]
    spec = np.zeros(stored_shape(fg["n"], half) + (ncomp,), dtype=np.complex128)
    pairs = [shared_slices(g["n"][d], fg["n"][d], d == half) for d in range(3)]
    for cx, fx in pairs[0]:
        for cy, fy in pairs[1]:
            for cz, fz in pairs[2]:
                spec[fx, fy, fz] = F[cx, cy, cz] * ratio
    phys = to_physical(spec, fg["n"], half)
    return window_gather(fg, phys, positions, W, beta, dtype)


def nufft_anterpolate(g, half, positions, q, W, beta, sigma=2, dtype=np.float64):
    """NUFFT type 1 (anterpolate with a NUFFT, alpha = 1, beta = 0)."""
    fg = _fine_grid(g, sigma)
    ratio = float(np.prod(fg["n"]) / np.prod(g["n"]))
    phys = window_spread(fg, positions, q, W, beta, dtype)
    spec = to_spectral(phys, half)
    out = np.zeros(stored_shape(g["n"], half) + (phys.shape[3],), dtype=np.complex128)
    pairs = [shared_slices(g["n"][d], fg["n"][d], d == half) for d in range(3)]
    for cx, fx in pairs[0]:
        for cy, fy in pairs[1]:
            for cz, fz in pairs[2]:
                out[cx, cy, cz] = spec[fx, fy, fz] / ratio
    D = deconvolution(g["n"], half, sigma, W, beta, dtype)
    return out * ratio * D[..., None]
