"""Seeded synthetic SLC pairs and GMTSAR PRM files.

The xcorr path reads two single-look-complex (SLC) images: row-major lines of
complex int16 I/Q samples (``read_complex_short2``, read_xcorr_data.c:11-29) or,
with ``-real``, float32 samples (``read_real_float2``, read_xcorr_data.c:31-49),
described by a PRM text file of ``key = value`` lines (``get_sio_struct``,
sio_struct.c:132-223).  This module writes both.

Speckle is i.i.d. complex Gaussian (I and Q ~ N(0, sigma^2)).  The aligned
(slave) image is the master delayed by (dx, dy) pixels,
``slave(x, y) = master(x - dx, y - dy)``, applied as a Fourier phase ramp,
plus complex Gaussian noise at ``noise_frac`` of the signal power, then
re-quantised to int16.  A feature at master pixel x therefore appears at
slave pixel x + dx.  All draws come from ``numpy.random.default_rng(seed)``.
"""
from __future__ import annotations

import hashlib
import os
from dataclasses import dataclass, field, asdict

import numpy as np


def speckle(nx: int, ny: int, sigma: float, rng: np.random.Generator) -> np.ndarray:
    """Complex Gaussian speckle, shape (ny, nx), complex128."""
    g = rng.standard_normal((ny, nx, 2))
    g *= sigma
    return g[..., 0] + 1j * g[..., 1]


def fourier_shift(z: np.ndarray, dx: float, dy: float) -> np.ndarray:
    """Delay a complex image by (dx, dy) pixels with a linear Fourier phase."""
    ny, nx = z.shape
    kx = np.fft.fftfreq(nx)
    ky = np.fft.fftfreq(ny)
    Z = np.fft.fft2(z)
    Z *= np.exp(-2j * np.pi * ky * dy)[:, None]
    Z *= np.exp(-2j * np.pi * kx * dx)[None, :]
    return np.fft.ifft2(Z)


def quantize_ci16(z: np.ndarray) -> np.ndarray:
    """Round and clip a complex image to interleaved int16 I/Q, shape (ny, nx, 2)."""
    out = np.empty(z.shape + (2,), dtype=np.int16)
    out[..., 0] = np.clip(np.rint(z.real), -32768, 32767)
    out[..., 1] = np.clip(np.rint(z.imag), -32768, 32767)
    return out


@dataclass
class PairSpec:
    """A synthetic pair: image size, constant shift, noise, seed."""
    nx: int
    ny: int
    dx: float
    dy: float
    noise_frac: float = 0.1
    sigma: float = 1000.0
    seed: int = 1
    real: bool = False            # write float32 real samples (the -real format)
    zero_rows: tuple = ()         # (r0, r1): master rows set to zero (edge cases)
    slave_nx: int | None = None   # slave width if different from the master
    slave_ny: int | None = None

    def to_dict(self):
        return asdict(self)


def make_pair(spec: PairSpec):
    """Return (master, slave) arrays.

    complex format: int16 arrays of shape (ny, nx, 2);
    real format: float32 arrays of shape (ny, nx) holding speckle amplitude.
    """
    rng = np.random.default_rng(spec.seed)
    m = speckle(spec.nx, spec.ny, spec.sigma, rng)
    mq = quantize_ci16(m)
    mz = mq[..., 0].astype(np.float64) + 1j * mq[..., 1].astype(np.float64)
    s = fourier_shift(mz, spec.dx, spec.dy)
    if spec.noise_frac > 0:
        s = s + speckle(spec.nx, spec.ny, spec.sigma * np.sqrt(spec.noise_frac), rng)
    sq = quantize_ci16(s)
    if spec.zero_rows:
        r0, r1 = spec.zero_rows
        mq[r0:r1] = 0
    snx = spec.slave_nx or spec.nx
    sny = spec.slave_ny or spec.ny
    if (snx, sny) != (spec.nx, spec.ny):
        out = np.zeros((sny, snx, 2), dtype=np.int16)
        h, w = min(sny, spec.ny), min(snx, spec.nx)
        out[:h, :w] = sq[:h, :w]
        sq = out
    if spec.real:
        ma = np.hypot(mq[..., 0].astype(np.float32), mq[..., 1].astype(np.float32)).astype(np.float32)
        sa = np.hypot(sq[..., 0].astype(np.float32), sq[..., 1].astype(np.float32)).astype(np.float32)
        return ma, sa
    return mq, sq


def sha256(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def write_prm(path: str, slc_file: str, nx: int, ny: int, rshift: int = 0, ashift: int = 0,
              prf: float = 1679.9):
    """Write the PRM keys xcorr reads (parse_xcorr_input.c:199-226, sio_struct.c:153-195)."""
    with open(path, "w") as f:
        f.write(f"SLC_file = {slc_file}\n")
        f.write(f"num_rng_bins = {nx}\n")
        f.write("num_patches = 1\n")
        f.write(f"num_valid_az = {ny}\n")
        f.write(f"rshift = {rshift}\n")
        f.write(f"ashift = {ashift}\n")
        f.write(f"PRF = {prf:.9f}\n")


def write_case(dirname: str, spec: PairSpec, rshift: int = 0, ashift: int = 0,
               prf_master: float = 1679.9, prf_slave: float | None = None):
    """Write master.SLC, aligned.SLC and their PRM files into ``dirname``.

    Returns (master_array, slave_array)."""
    os.makedirs(dirname, exist_ok=True)
    m, s = make_pair(spec)
    m.tofile(os.path.join(dirname, "master.SLC"))
    s.tofile(os.path.join(dirname, "aligned.SLC"))
    write_prm(os.path.join(dirname, "master.PRM"), "master.SLC", m.shape[1], m.shape[0], 0, 0, prf_master)
    write_prm(os.path.join(dirname, "aligned.PRM"), "aligned.SLC", s.shape[1], s.shape[0], rshift, ashift,
              prf_slave if prf_slave is not None else prf_master)
    return m, s


def make_pair_varying(nx: int, ny: int, shift_fn, noise_frac: float, sigma: float = 1000.0, seed: int = 2,
                      tile: int = 512, margin: int = 64, device=None):
    """Speckle pair with a spatially varying shift, generated with torch.

    shift_fn(x, y) -> (dx, dy) in pixels, evaluated at the centre of each
    tile x tile block; each block of the slave is the master delayed by that
    block's shift (Fourier phase ramp over the block plus `margin` pixels on
    every side, wrapped at the image border), so the truth is piecewise
    constant: ``truth(x, y)`` returns the shift of the block holding (x, y).
    Noise: complex Gaussian at `noise_frac` of the signal power.  Returns
    (master, slave, truth) with int16 arrays of shape (ny, nx, 2) (numpy);
    device: a torch device for the transforms (default: cuda if available)."""
    import torch
    if device is None:
        device = torch.device("cuda" if torch.cuda.is_available() else "cpu")
    g = torch.Generator(device="cpu").manual_seed(seed)
    m = torch.randn((ny, nx, 2), generator=g, dtype=torch.float32).mul_(sigma).round_().clamp_(-32768, 32767)
    master = m.to(torch.int16)
    mz = torch.complex(m[..., 0], m[..., 1]).to(device)
    out = torch.empty((ny, nx), dtype=torch.complex64, device=device)
    P = tile + 2 * margin
    k = torch.fft.fftfreq(P, device=device, dtype=torch.float64)
    for y0 in range(0, ny, tile):
        for x0 in range(0, nx, tile):
            th, tw_ = min(tile, ny - y0), min(tile, nx - x0)
            dx, dy = shift_fn(x0 + tw_ / 2.0, y0 + th / 2.0)
            ys = (torch.arange(y0 - margin, y0 - margin + P, device=device) % ny)
            xs = (torch.arange(x0 - margin, x0 - margin + P, device=device) % nx)
            blk = mz[ys][:, xs].to(torch.complex128)
            B = torch.fft.fft2(blk)
            ramp = torch.exp(-2j * torch.pi * (k[:, None] * dy + k[None, :] * dx))
            sb = torch.fft.ifft2(B * ramp)
            out[y0:y0 + th, x0:x0 + tw_] = sb[margin:margin + th, margin:margin + tw_].to(torch.complex64)
    nz = torch.randn((ny, nx, 2), generator=g, dtype=torch.float32).mul_(sigma * float(np.sqrt(noise_frac)))
    nz = nz.to(device)
    sr = (out.real + nz[..., 0]).round_().clamp_(-32768, 32767)
    si = (out.imag + nz[..., 1]).round_().clamp_(-32768, 32767)
    slave = torch.stack([sr, si], dim=-1).to(torch.int16).cpu()

    def truth(x, y):
        bx = (np.asarray(x) // tile) * tile
        by = (np.asarray(y) // tile) * tile
        cx = bx + np.minimum(tile, nx - bx) / 2.0
        cy = by + np.minimum(tile, ny - by) / 2.0
        return shift_fn(cx, cy)

    return master.numpy(), slave.numpy(), truth


def cfg2_shift(x, y):
    """The full-frame configuration's shift field (px): dx = 2.1 + 1e-5 x - 3e-6 y,
    dy = -4.7 + 2e-6 x + 8e-6 y."""
    return 2.1 + 1e-5 * np.asarray(x) - 3e-6 * np.asarray(y), -4.7 + 2e-6 * np.asarray(x) + 8e-6 * np.asarray(y)
