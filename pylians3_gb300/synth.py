"""Seeded synthetic particle sets of the benchmark workloads, made on the GPU.

* ``uniform(n, BoxSize, seed)``: i.i.d. uniform float32 positions in
  [0, BoxSize).
* ``zeldovich(dims, BoxSize, sigma, seed, rsd=0.5)``: a regular lattice of
  dims^3 particles (cell centres) displaced by the Zel'dovich displacement of
  a Gaussian random field with P(k) = A k^-1.5 exp(-(k/0.5)^2) (k in h/Mpc),
  A set so that the rms displacement per component is ``sigma`` Mpc/h; then
  a redshift-space shift z += rsd * psi_z and a periodic wrap into
  [0, BoxSize), as library/redshift_space_library wraps positions.
* ``plummer_halos(n, nhalos, scale, BoxSize, seed)``: particles in Plummer
  spheres around uniformly placed centres, periodically wrapped.
The Fourier transforms use this package's own c2r FFT (IFFT3Dr_f).
"""
from __future__ import annotations

import math


def _gen(seed, device):
    import torch
    return torch.Generator(device=device).manual_seed(int(seed))


def uniform(n, BoxSize, seed=0, device="cuda"):
    import torch
    g = _gen(seed, device)
    pos = torch.rand((int(n), 3), generator=g, device=device, dtype=torch.float32)
    pos.mul_(float(BoxSize))
    # rand * BoxSize can round up to BoxSize itself; keep [0, BoxSize)
    pos.clamp_(max=math.nextafter(float(BoxSize), 0.0))
    return pos


def zeldovich(dims, BoxSize, sigma=3.0, seed=0, rsd=0.5, device="cuda"):
    import torch
    from . import Pk_library as PKL

    dims = int(dims)
    g = _gen(seed, device)
    noise = torch.randn((dims,) * 3, generator=g, device=device, dtype=torch.float32)
    dk = PKL.FFT3Dr_f(noise, 1)                       # (d, d, d/2+1) complex64
    del noise
    kF = 2.0 * math.pi / BoxSize
    f = torch.fft.fftfreq(dims, d=1.0 / dims, device=device).to(torch.float32)  # integers
    fz = torch.arange(dims // 2 + 1, device=device, dtype=torch.float32)
    kx, ky, kz = f.view(-1, 1, 1), f.view(1, -1, 1), fz.view(1, 1, -1)
    k2 = (kx * kx + ky * ky + kz * kz) * (kF * kF)
    k2[0, 0, 0] = 1.0
    kmag = torch.sqrt(k2)
    amp = torch.pow(kmag, -0.75) * torch.exp(-0.5 * (kmag / 0.5) ** 2)
    amp[0, 0, 0] = 0.0
    dk.mul_(amp)
    del amp, kmag
    psi = []
    for kc in (kx, ky, kz):
        comp = dk * (1j * (kc * kF) / k2)             # psi_i(k) = i k_i / k^2 delta(k)
        psi.append(PKL.IFFT3Dr_f(comp.to(torch.complex64).contiguous(), 1))
        del comp
    del dk, k2
    rms = math.sqrt(sum(float(p.double().pow(2).mean()) for p in psi) / 3.0)
    scale = float(sigma) / rms
    cell = BoxSize / dims
    lat = (torch.arange(dims, device=device, dtype=torch.float32) + 0.5) * cell
    pos = torch.empty((dims ** 3, 3), device=device, dtype=torch.float32)
    pos[:, 0] = (lat.view(-1, 1, 1) + psi[0] * scale).reshape(-1)
    pos[:, 1] = (lat.view(1, -1, 1) + psi[1] * scale).reshape(-1)
    pos[:, 2] = (lat.view(1, 1, -1) + psi[2] * scale * (1.0 + rsd)).reshape(-1)
    del psi
    pos.remainder_(float(BoxSize))
    pos.clamp_(min=0.0, max=math.nextafter(float(BoxSize), 0.0))
    return pos


def plummer_halos(n, nhalos, scale, BoxSize, seed=0, device="cuda"):
    import torch
    g = _gen(seed, device)
    centres = torch.rand((int(nhalos), 3), generator=g, device=device) * BoxSize
    which = torch.randint(0, int(nhalos), (int(n),), generator=g, device=device)
    # Plummer radius from the inverse cumulative mass: r = a / sqrt(u^(-2/3) - 1)
    u = torch.rand((int(n),), generator=g, device=device).clamp_(1e-6, 1 - 1e-6)
    r = scale / torch.sqrt(torch.pow(u, -2.0 / 3.0) - 1.0)
    r.clamp_(max=50.0 * scale)
    d = torch.randn((int(n), 3), generator=g, device=device)
    d = d / d.norm(dim=1, keepdim=True).clamp_(min=1e-12)
    pos = centres[which] + d * r.unsqueeze(1)
    pos.remainder_(float(BoxSize))
    pos.clamp_(min=0.0, max=math.nextafter(float(BoxSize), 0.0))
    return pos.to(torch.float32)
