"""PML damping profile (seistorch/pml.py:29-59)."""
import math

import torch


def generate_pml_coefficients_2d(domain_shape, N=50, B=100., multiple=False):
    """d(z, x): d0 = 1.5*1500/N*log10(1e4), a quadratic ramp over N+1 cells
    on each side (d0 at the outer cell, 0 at cell N), sqrt(dz^2 + dx^2) in
    the corners, no top ramp with ``multiple``.  Torch default dtype."""
    nz, nx = domain_shape
    dz = torch.zeros(nz, nx)
    dx = torch.zeros(nz, nx)
    if N > 0:
        d0 = (1.5 * 1500.0 / N) * math.log10(1e4)
        ramp = torch.flip(d0 * torch.linspace(0.0, 1.0, N + 1) ** 2, [0])
        dx[:, 0:N + 1] = ramp[None, :]
        dx[:, nx - N - 1:nx] = torch.flip(ramp, [0])[None, :]
        if not multiple:
            dz[0:N + 1, :] = ramp[:, None]
        dz[nz - N - 1:nz, :] = torch.flip(ramp, [0])[:, None]
    return torch.sqrt(dz ** 2 + dx ** 2)
