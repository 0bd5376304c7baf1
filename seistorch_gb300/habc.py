"""HABC strip masks and blend weights (seistorch/habc.py:4-81)."""
import torch


def bound_mask(nz, nx, w, dev="cpu", batchsize=1, return_idx=False, multiple=False):
    """Strip masks top (w, nx), bottom (w, nx), left (nz, w), right (nz, w):
    top[r, x] = r <= x <= nx-1-r; left[z, c] = c <= z and c <= nz-1-z (rows
    z < w all set with ``multiple``, which also drops the top mask); bottom
    and right are the mirror images.  ``return_idx`` gives boolean masks,
    repeated over the batch when batchsize > 1."""
    r = torch.arange(w, device=dev)[:, None]
    x = torch.arange(nx, device=dev)[None, :]
    top = ((x >= r) & (x <= nx - 1 - r)).to(torch.get_default_dtype())
    bottom = torch.flipud(top)
    z = torch.arange(nz, device=dev)[:, None]
    c = torch.arange(w, device=dev)[None, :]
    zf = nz - 1 - z
    left = (~((z < w) & (c > z)) & ~((zf < w) & (c > zf))).to(torch.get_default_dtype())
    right = torch.fliplr(left)
    if multiple:
        top = None
        left[:w] = 1.0
        right[:w] = 1.0
    if not return_idx:
        return top, bottom, left, right
    if batchsize > 1:
        rep = lambda m: None if m is None else m.repeat(batchsize, 1, 1) == 1
    else:
        rep = lambda m: None if m is None else m == 1
    return rep(top), rep(bottom), rep(left), rep(right)


def generate_habc_coefficients_2d(domain_shape, N=50, multiple=False, device="cpu"):
    """Blend weight b(z, x): (N-1-k)/(N-1) at depth k from each side, written
    top, bottom, left, right through the masks (later sides win)."""
    nz, nx = domain_shape
    d = torch.zeros(nz, nx, device=device)
    if N <= 0:
        return d
    dv = torch.flip(torch.linspace(0.0, N, N, device=device) / N, [0])
    tm, bm, lm, rm = bound_mask(nz, nx, N, device, multiple=multiple)
    if not multiple:
        idx = tm == 1
        d[:N][idx] = dv[:, None].expand(N, nx)[idx]
    idx = bm == 1
    d[-N:][idx] = torch.flip(dv, [0])[:, None].expand(N, nx)[idx]
    idx = lm == 1
    d[:, :N][idx] = dv[None, :].expand(nz, N)[idx]
    idx = rm == 1
    d[:, -N:][idx] = torch.flip(dv, [0])[None, :].expand(nz, N)[idx]
    return d
