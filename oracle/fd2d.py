"""Numpy restatement of seistorch's 2D acoustic / elastic time stepping.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Every function cites the reference file:line it restates (paths inside the
seistorch project).  Arrays are (Nz, Nx) for models and (B, Nz, Nx) for
wavefields; ``dtype`` selects the arithmetic (float64 for the oracle, float32
for the CPU baseline).
"""
import numpy as np

# ---------------------------------------------------------------- setup ---


def fd_coefficients(order):
    """Second-derivative Taylor weights c_1..c_M, M = order/2.

    Restates ``even_intergrid`` (equations2d/acoustic.py:5-30): solve
    sum_j c_j j^(2i) = [i == 0] for i < M (the weights of
    u(x+j)+u(x-j)), then divide by j^2.  Order 2 -> [1], order 4 ->
    [4/3, -1/12].
    """
    if order < 2 or order % 2:
        raise ValueError(f"spatial order must be an even integer >= 2, got {order}")
    m = order // 2
    a = np.array([[float(j + 1) ** (2 * i) for j in range(m)] for i in range(m)])
    rhs = np.zeros(m)
    rhs[0] = 1.0
    c = np.linalg.solve(a, rhs)
    return c / np.array([(j + 1) ** 2 for j in range(m)], dtype=np.float64)


def laplacian_kernel(order):
    """(order+1)^2 cross stencil; centre = -4 sum(c)  (acoustic.py:32-53)."""
    c = fd_coefficients(order)
    r = order // 2
    k = np.zeros((order + 1, order + 1))
    k[r, r + 1:] = c
    k[r, :r] = c[::-1]
    k[r + 1:, r] = c
    k[:r, r] = c[::-1]
    k[r, r] = -4.0 * c.sum()
    return k


def pml_profile_2d(shape, N=50, multiple=False, dtype=np.float64):
    """Damping profile d(z, x) (pml.py:29-59).

    d0 = 1.5*1500/N*log10(1e4); per side a quadratic ramp over N+1 cells
    (d0 at the outer edge, 0 at cell N); corners combine as
    sqrt(dz^2 + dx^2); the top side is absent when ``multiple``.  The
    reference computes this in torch's default dtype; ``dtype`` plays
    that role here.
    """
    nz, nx = shape
    d0 = (1.5 * 1500.0 / N) * np.log10(1e4) if N > 0 else 0.0
    ramp = (d0 * np.linspace(0.0, 1.0, N + 1, dtype=dtype) ** 2)[::-1].astype(dtype)
    dz = np.zeros((nz, nx), dtype)
    dx = np.zeros((nz, nx), dtype)
    if N > 0:
        # pml.py:36-54 unpacks (nz, nx) as "Nx, Ny" and transposes at the
        # end: its first array ramps along x at both sides, its second along
        # z, whose top ramp is the one dropped for ``multiple``.
        dx[:, 0:N + 1] = ramp[None, :]
        dx[:, nx - N - 1:nx] = ramp[::-1][None, :]
        if not multiple:
            dz[0:N + 1, :] = ramp[:, None]
        dz[nz - N - 1:nz, :] = ramp[::-1][:, None]
    return np.sqrt(dz ** 2 + dx ** 2).astype(dtype)


def habc_masks(nz, nx, w=50, multiple=False):
    """Boolean strip masks (top, bottom, left, right) (habc.py:4-40).

    top[r, x]  (r < w):  r <= x <= nx-1-r      (None when ``multiple``)
    bottom: top mirrored in z; left[z, c] (c < w): c <= z and c <= nz-1-z,
    with rows z < w all set when ``multiple``; right: left mirrored in x.
    """
    r = np.arange(w)[:, None]
    x = np.arange(nx)[None, :]
    top = (x >= r) & (x <= nx - 1 - r)
    bottom = top[::-1].copy()
    z = np.arange(nz)[:, None]
    c = np.arange(w)[None, :]
    first = ~((z < w) & (c > z))
    zf = nz - 1 - z
    second = ~((zf < w) & (c > zf))
    left = first & second
    right = left[:, ::-1].copy()
    if multiple:
        left[:w] = True
        right[:w] = True
        top = None
    return top, bottom, left, right


def habc_coefficients_2d(shape, N=50, multiple=False, dtype=np.float64):
    """HABC blend weight b(z, x) (habc.py:42-81).

    Along each side the weight falls linearly from 1 at the outer cell to 0
    at cell N-1: d_vals[k] = (N-1-k)/(N-1) (torch.linspace(0,N,N)/N
    flipped, in torch's default dtype -- ``dtype`` here).  Written side by
    side in the order top, bottom, left, right through the masks of
    ``habc_masks`` (later sides win).
    """
    nz, nx = shape
    d = np.zeros((nz, nx), dtype)
    if N <= 0:
        return d
    dv = (np.linspace(0.0, N, N, dtype=dtype) / dtype(N))[::-1].astype(dtype)
    tm, bm, lm, rm = habc_masks(nz, nx, N, multiple)
    if not multiple:
        blk = np.repeat(dv[:, None], nx, 1)
        d[:N][tm] = blk[tm]
    blk = np.repeat(dv[::-1][:, None], nx, 1)
    d[-N:][bm] = blk[bm]
    blk = np.repeat(dv[None, :], nz, 0)
    d[:, :N][lm] = blk[lm]
    blk = np.repeat(dv[::-1][None, :], nz, 0)
    d[:, -N:][rm] = blk[rm]
    return d


def ricker(fm, dt, T, delay=80, inverse=False):
    """Ricker wavelet, rounded to float32 (utils.py:235-249)."""
    i = np.arange(T, dtype=np.float64)
    c = np.pi * fm * (i * dt - delay * dt)
    p = -1.0 if inverse else 1.0
    return (p * (1 - 2 * c ** 2) * np.exp(-c ** 2)).astype(np.float32)


def pad_model(m, width, multiple=False):
    """Edge padding by the boundary width, top unpadded with ``multiple``
    (geom.py:213-240)."""
    top = 0 if multiple else width
    return np.pad(m, ((top, width), (width, width)), mode="edge")


# ------------------------------------------------------------ stencils ---


def laplacian(u, order, h, dtype=np.float64):
    """Zero-padded cross-stencil Laplacian / h^2 of (B, Nz, Nx) fields
    (acoustic.py:60-71, conv2d with padding=order/2)."""
    u = np.asarray(u, dtype)
    c = fd_coefficients(order).astype(dtype)
    r = order // 2
    nz, nx = u.shape[-2:]
    up = np.pad(u, ((0, 0), (r, r), (r, r)))
    out = dtype(-4.0 * fd_coefficients(order).sum()) * u
    for j in range(1, r + 1):
        out = out + c[j - 1] * (up[:, r + j:r + j + nz, r:r + nx] + up[:, r - j:r - j + nz, r:r + nx]
                                + up[:, r:r + nz, r + j:r + j + nx] + up[:, r:r + nz, r - j:r - j + nx])
    return out * dtype(1.0 / (h * h))


def acoustic_step(vp, h1, h2, dt, h, d, order, dtype=np.float64):
    """One 2nd-order acoustic PML step (acoustic.py:73-86).

    y = (dt^-2 + d/dt)^-1 (2/dt^2 h1 - (dt^-2 - d/dt) h2 + vp^2 lap(h1));
    returns (y, h1).
    """
    vp = np.asarray(vp, dtype)
    d = np.asarray(d, dtype)
    dt = dtype(dt)
    lap = laplacian(h1, order, h, dtype)
    y = (dt ** -2 + d / dt) ** -1 * (2 / dt ** 2 * h1 - (dt ** -2 - d / dt) * h2 + vp ** 2 * lap)
    return y.astype(dtype), np.asarray(h1, dtype)


def _one_way(u_now, u_pre, y, c, b, dt, h, depth_axis, from_end, w=50):
    """HABC one-way extrapolation + blend for one side, over the 50-cell
    strip (acoustic_habc.py:79-101).

    Depth k counts cells from the outer edge.  With U(k) = u_now at depth k:
      u_one = (2-lam-mu) U(k) + (lam+2mu) U(k+1) - mu U(k+2)
              + (lam-1) P(k) - lam P(k+1),    lam = 2c dt/h, mu = c^2 dt^2/h^2
    and the result is b*u_one + (1-b)*y.  The reference builds a 51-deep
    slab and uses torch.roll, so U(k+2) at k = 49 wraps to depth 0
    (acoustic_habc.py:93-96); that wrap is kept.
    Returns an array of the strip's shape (w along depth_axis).
    """
    n = u_now.shape[depth_axis]

    def take(a, k):
        idx = (n - 1 - k) if from_end else k
        return np.take(a, idx, axis=depth_axis)

    out = []
    for k in range(w):
        k2 = (k + 2) if (k + 2) <= w else (k + 2) - (w + 1)
        cc = take(c, k)
        bb = take(b, k)
        lam = 2 * cc * dt / h
        mu = cc ** 2 * dt ** 2 / h ** 2
        uo = ((2 - lam - mu) * take(u_now, k) + (lam + 2 * mu) * take(u_now, k + 1)
              - mu * take(u_now, k2) + (lam - 1) * take(u_pre, k) - lam * take(u_pre, k + 1))
        out.append(uo * bb + (1 - bb) * take(y, k))
    st = np.stack(out, axis=depth_axis)
    if from_end:
        st = np.flip(st, axis=depth_axis)
    return st


def habc_apply(y, h1, h2, vp, b, dt, h, w=50, multiple=False, dtype=np.float64):
    """Hybrid ABC on the four strips (acoustic_habc.py:147-204).

    Strip results are scattered through the masks in the order top,
    bottom, left, right (later sides win), then four 50-cell diagonals are
    replaced by 0.5/0.5 averages: (i, i) top/left, (i, nx-w+i) top/right,
    (nz-w+i, i) bottom/left, (nz-w+i, nx-w+i) bottom/right (the top ones
    are skipped with ``multiple``).
    """
    y = np.array(y, dtype)
    h1 = np.asarray(h1, dtype)
    h2 = np.asarray(h2, dtype)
    vp = np.asarray(vp, dtype)[None]
    b = np.asarray(b, dtype)[None]
    dt = dtype(dt)
    h = dtype(h)
    nz, nx = y.shape[-2:]
    tm, bm, lm, rm = habc_masks(nz, nx, w, multiple)
    yt = _one_way(h1, h2, y, vp, b, dt, h, 1, False, w)       # (B, w, nx) rows 0..w-1
    yb = _one_way(h1, h2, y, vp, b, dt, h, 1, True, w)        # rows nz-w..nz-1
    yl = _one_way(h1, h2, y, vp, b, dt, h, 2, False, w)       # cols 0..w-1
    yr = _one_way(h1, h2, y, vp, b, dt, h, 2, True, w)        # cols nx-w..nx-1
    out = y.copy()
    if not multiple:
        out[:, :w, :][:, tm] = yt[:, tm]
    out[:, -w:, :][:, bm] = yb[:, bm]
    out[:, :, :w][:, lm] = yl[:, lm]
    out[:, :, -w:][:, rm] = yr[:, rm]
    i = np.arange(w)
    half = dtype(0.5)
    if not multiple:
        out[:, i, i] = half * yt[:, i, i] + half * yl[:, i, i]
        out[:, i, nx - w + i] = half * yt[:, i, nx - w + i] + half * yr[:, i, i]
    out[:, nz - w + i, i] = half * yb[:, i, i] + half * yl[:, nz - w + i, i]
    out[:, nz - w + i, nx - w + i] = half * yb[:, i, nx - w + i] + half * yr[:, nz - w + i, i]
    return out


def acoustic_habc_step(vp, h1, h2, dt, h, b, order, multiple=False, dtype=np.float64):
    """Undamped interior step then HABC (acoustic_habc.py:206-221)."""
    vp = np.asarray(vp, dtype)
    dt_ = dtype(dt)
    lap = laplacian(h1, order, h, dtype)
    y = (dt_ ** -2) ** -1 * (2 / dt_ ** 2 * np.asarray(h1, dtype) - dt_ ** -2 * np.asarray(h2, dtype)
                             + vp ** 2 * lap)
    y = habc_apply(y, h1, h2, vp, b, dt, h, 50, multiple, dtype)
    return y, np.asarray(h1, dtype)


def born_habc_step(vp, m, h1, h2, sh1, sh2, dt, h, b, order, multiple=False, dtype=np.float64):
    """Born modelling step (acoustic_lsrtm_habc.py:11-30): background
    p0 = 2 h1 - h2 + vp^2 lap(h1) dt^2, scattered
    sh0 = 2 sh1 - sh2 + vp^2 lap(sh1) dt^2 + m vp^2 lap(h1) dt^2, each then
    blended by the HABC of its own field.  Returns (p0, h1, sh0, sh1)."""
    vp = np.asarray(vp, dtype)
    m = np.asarray(m, dtype)
    dt_ = dtype(dt)
    vp2_lap_p = vp ** 2 * laplacian(h1, order, h, dtype)
    p0 = 2 * np.asarray(h1, dtype) - np.asarray(h2, dtype) + vp2_lap_p * dt_ ** 2
    s0 = (2 * np.asarray(sh1, dtype) - np.asarray(sh2, dtype) + vp ** 2 * laplacian(sh1, order, h, dtype) * dt_ ** 2
          + m * vp2_lap_p * dt_ ** 2)
    p0 = habc_apply(p0, h1, h2, vp, b, dt, h, 50, multiple, dtype)
    s0 = habc_apply(s0, sh1, sh2, vp, b, dt, h, 50, multiple, dtype)
    return p0, np.asarray(h1, dtype), s0, np.asarray(sh1, dtype)


def vacoustic_habc_step(vp, Q, h1, h2, dt, h, b, order=2, multiple=False, omega=16.5, dtype=np.float64):
    """Viscoacoustic step with HABC (vacoustic_habc.py:74-115):
    y = 2 h1 - h2 + vp^2 dt^2 (1 - (1 - sqrt(Q^2 + 1)) / Q^2) lap(h1)
        - (dt^2 t vp / 2) real(ifft2(|k| fft2((h1 - h2) / dt))),
    |k| = sqrt(kz^2 + kx^2) from fftfreq(nz, h) and fftfreq(nx, h); t from Q
    and omega: t_sigma = (sqrt(1 + Q^-2) - 1/Q) / omega, t_eps =
    1 / (omega^2 t_sigma), t = t_eps / (t_sigma - 1e-8) - 1; then the HABC
    blend.  Returns (y, h1)."""
    vp = np.asarray(vp, dtype)
    Q = np.asarray(Q, dtype)
    h1 = np.asarray(h1, dtype)
    h2 = np.asarray(h2, dtype)
    dt_ = dtype(dt)
    t_sigma = (np.sqrt(1 + Q ** -2) - Q ** -1) / omega
    t_eps = 1.0 / (omega ** 2 * t_sigma)
    t = t_eps / (t_sigma - 1e-8) - 1.0
    lap = laplacian(h1, order, h, dtype)
    y = 2 * h1 - h2 + vp ** 2 * dt_ ** 2 * (1 - (1 - np.sqrt(Q ** 2 + 1)) * Q ** -2) * lap
    nz, nx = h1.shape[-2:]
    kz, kx = np.meshgrid(np.fft.fftfreq(nz, d=h), np.fft.fftfreq(nx, d=h), indexing="ij")
    k = np.sqrt(kz ** 2 + kx ** 2)
    dy = (h1 - h2) / dt_
    temp = np.real(np.fft.ifft2(k * np.fft.fft2(dy, axes=(-2, -1)), axes=(-2, -1)))
    y = y - (dt_ ** 2 * t * vp / 2) * temp
    y = habc_apply(y, h1, h2, vp, b, dt, h, 50, multiple, dtype)
    return y, h1


def second_difference(u, axis, h, dtype=np.float64):
    """Zero-padded 1-D second difference / h^2 along `axis` of (B, Nz, Nx)
    fields (convkernel.py kernelx / kernely at spatial order 2: [1, -2, 1])."""
    u = np.asarray(u, dtype)
    up = np.pad(u, [(0, 0)] + [(1, 1) if ax == axis % 3 else (0, 0) for ax in (1, 2)])
    n = u.shape[axis]
    lo = np.take(up, np.arange(0, n), axis=axis)
    hi = np.take(up, np.arange(2, n + 2), axis=axis)
    return (lo + hi - 2 * u) * dtype(1.0 / (h * h))


def vti_sk(eps, delta, h, dtype=np.float64):
    """The reference's per-cell sk (vti_habc2.py:36-45): fftfreq of the rows
    (named kx there) and columns (kz), meshgrid 'ij'."""
    eps = np.asarray(eps, dtype)
    delta = np.asarray(delta, dtype)
    nz, nx = eps.shape
    fx = np.fft.fftfreq(nz, d=h).astype(dtype)
    fz = np.fft.fftfreq(nx, d=h).astype(dtype)
    kx, kz = np.meshgrid(fx, fz, indexing="ij")
    num = -2 * (eps - delta) * kx ** 2 * kz ** 2
    den = (1 + 2 * eps) * kx ** 4 + kz ** 4 + 2 * (1 + delta) * kx ** 2 * kz ** 2
    return num * (den + dtype(1e-26)) ** -1


def vti_habc_step(vp, eps, delta, p1, p2, dt, h, b, multiple=False, dtype=np.float64):
    """VTI step (vti_habc2.py:26-56): 2 p1 - p2 + vp^2 dt^2 ((1 + 2 eps) + sk)
    d2x(p1) + vp^2 dt^2 (1 + sk) d2z(p1), then the HABC blend (with vp).
    Returns (pnext, p1)."""
    vp = np.asarray(vp, dtype)
    eps = np.asarray(eps, dtype)
    sk = vti_sk(eps, delta, h, dtype)
    v2 = vp ** 2 * dtype(dt) ** 2
    p1 = np.asarray(p1, dtype)
    y = (2 * p1 - np.asarray(p2, dtype) + v2 * ((1 + 2 * eps) + sk) * second_difference(p1, 2, h, dtype)
         + v2 * (1 + sk) * second_difference(p1, 1, h, dtype))
    y = habc_apply(y, p1, p2, vp, b, dt, h, 50, multiple, dtype)
    return y, p1


def rho_habc_step(vp, rho, p1, p2, dt, h, b, multiple=False, dtype=np.float64):
    """Variable-density step (acoustic_rho_habc.py:34-58): one-cell forward /
    backward differences of p1 and buoyancy averages of 1/rho, all with the
    zero padding of the reference's conv2d, then the HABC blend (with vp).
    Returns (pnext, p1)."""
    vp = np.asarray(vp, dtype)
    rho = np.asarray(rho, dtype)
    p1 = np.asarray(p1, dtype)
    bu = 1 / rho
    pp = np.pad(p1, ((0, 0), (1, 1), (1, 1)))
    bp = np.pad(bu, 1)
    pxp = pp[:, 1:-1, 2:] - p1
    pxn = p1 - pp[:, 1:-1, :-2]
    pzp = pp[:, 2:, 1:-1] - p1
    pzn = p1 - pp[:, :-2, 1:-1]
    bxp = (bu + bp[1:-1, 2:]) / 2
    bxn = (bp[1:-1, :-2] + bu) / 2
    bzp = (bu + bp[2:, 1:-1]) / 2
    bzn = (bp[:-2, 1:-1] + bu) / 2
    y = 2 * p1 - np.asarray(p2, dtype) + dtype(dt) ** 2 * dtype(h) ** -2 * rho * vp ** 2 * (
        bxp * pxp - bxn * pxn + bzp * pzp - bzn * pzn)
    y = habc_apply(y, p1, p2, vp, b, dt, h, 50, multiple, dtype)
    return y, p1


def dfwd(a, axis):
    """a[i] - a[i-1], zero at index 0 (equations2d/utils.py:3-25, forward)."""
    out = a - np.roll(a, 1, axis=axis)
    idx = [slice(None)] * a.ndim
    idx[axis] = 0
    out[tuple(idx)] = 0
    return out


def dbwd(a, axis):
    """a[i+1] - a[i], zero at the last index (equations2d/utils.py:27-43)."""
    out = np.roll(a, -1, axis=axis) - a
    idx = [slice(None)] * a.ndim
    idx[axis] = -1
    out[tuple(idx)] = 0
    return out


def elastic_step(vp, vs, rho, vx, vz, txx, tzz, txz, dt, h, d, dtype=np.float64):
    """Velocity-stress staggered step (elastic.py:7-37): stresses first
    (A-8..A-10), then velocities from the new stresses; c = 0.5 dt d."""
    vp, vs, rho, d = (np.asarray(a, dtype) for a in (vp, vs, rho, d))
    vx, vz, txx, tzz, txz = (np.asarray(a, dtype) for a in (vx, vz, txx, tzz, txz))
    dt = dtype(dt)
    h = dtype(h)
    lam = rho * (vp ** 2 - 2 * vs ** 2)
    mu = rho * vs ** 2
    c = dtype(0.5) * dt * d
    vx_x = dfwd(vx, 2)
    vz_z = dbwd(vz, 1)
    vx_z = dfwd(vx, 1)
    vz_x = dbwd(vz, 2)
    ytxx = (1 + c) ** -1 * (dt / h * ((lam + 2 * mu) * vx_x + lam * vz_z) + (1 - c) * txx)
    ytzz = (1 + c) ** -1 * (dt / h * ((lam + 2 * mu) * vz_z + lam * vx_x) + (1 - c) * tzz)
    ytxz = (1 + c) ** -1 * (dt * mu / h * (vz_x + vx_z) + (1 - c) * txz)
    txx_x = dbwd(ytxx, 2)
    txz_z = dbwd(ytxz, 1)
    tzz_z = dfwd(ytzz, 1)
    txz_x = dfwd(ytxz, 2)
    yvx = (1 + c) ** -1 * (dt / rho / h * (txx_x + txz_z) + (1 - c) * vx)
    yvz = (1 + c) ** -1 * (dt / rho / h * (txz_x + tzz_z) + (1 - c) * vz)
    return yvx, yvz, ytxx, ytzz, ytxz


# ----------------------------------------------------------- time loop ---

WAVEFIELDS = {"acoustic": ["h1", "h2"], "acoustic_habc": ["h1", "h2"],
              "acoustic_lsrtm_habc": ["h1", "h2", "sh1", "sh2"], "vti_habc2": ["p1", "p2"],
              "acoustic_rho_habc": ["h1", "h2"], "vacoustic_habc": ["h1", "h2"],
              "elastic": ["vx", "vz", "txx", "tzz", "txz"]}
MODEL_PARAMS = {"acoustic": ["vp"], "acoustic_habc": ["vp"], "acoustic_lsrtm_habc": ["vp", "m"],
                "vti_habc2": ["vp", "epsilon", "delta"], "acoustic_rho_habc": ["vp", "rho"],
                "vacoustic_habc": ["vp", "Q"], "elastic": ["vp", "vs", "rho"]}


def forward(equation, models, d, dt, h, wavelet, sources, receivers, *,
            order=2, multiple=False, source_type=None, receiver_type=None,
            illumination=False, dtype=np.float64, nt=None, return_fields=False):
    """Time loop of ``WaveRNN.forward`` (rnn.py:100-217).

    sources:   per shot, a list of (z, x) padded-grid points (the mask
               ``smask[b, z, x] = 1`` of rnn.py:158-166, so repeated points
               inject once);
    receivers: per shot, (zs, xs) index lists (probe.py:42-44).
    Per step: equation step; ``field[b, z, x] += w[i]`` at the shot's source
    points for every source_type (source.py:47-57, one shared wavelet
    value); records read every receiver_type after injection; the
    illumination adds sum_b src_field^2 (rnn.py:204-205).
    Returns dict(records=[(nt, nrec_b, nch)], fields=..., illum=...).
    """
    wavelet = np.asarray(wavelet, np.float64)
    nt = len(wavelet) if nt is None else nt
    names = WAVEFIELDS[equation]
    first = WAVEFIELDS[equation][0]
    source_type = source_type or ([first] if equation != "elastic" else ["txx", "tzz"])
    receiver_type = receiver_type or ([first] if equation != "elastic" else ["vx", "vz"])
    B = len(sources)
    m0 = np.asarray(models[MODEL_PARAMS[equation][0]])
    nz, nx = m0.shape
    fields = {n: np.zeros((B, nz, nx), dtype) for n in names}
    smask = np.zeros((B, nz, nx), dtype)
    for b, pts in enumerate(sources):
        for (z, x) in pts:
            smask[b, z, x] = 1
    recs = [[] for _ in range(B)]
    illum = np.zeros((nz, nx), dtype) if illumination else None
    for i in range(nt):
        if equation == "acoustic":
            y, h1 = acoustic_step(models["vp"], fields["h1"], fields["h2"], dt, h, d, order, dtype)
            fields["h1"], fields["h2"] = y, h1
        elif equation == "acoustic_habc":
            y, h1 = acoustic_habc_step(models["vp"], fields["h1"], fields["h2"], dt, h, d, order,
                                       multiple, dtype)
            fields["h1"], fields["h2"] = y, h1
        elif equation == "acoustic_lsrtm_habc":
            out = born_habc_step(models["vp"], models["m"], fields["h1"], fields["h2"], fields["sh1"],
                                 fields["sh2"], dt, h, d, order, multiple, dtype)
            fields = dict(zip(names, out))
        elif equation == "acoustic_rho_habc":
            y, h1 = rho_habc_step(models["vp"], models["rho"], fields["h1"], fields["h2"], dt, h, d, multiple, dtype)
            fields["h1"], fields["h2"] = y, h1
        elif equation == "vacoustic_habc":
            y, h1 = vacoustic_habc_step(models["vp"], models["Q"], fields["h1"], fields["h2"], dt, h, d, order,
                                        multiple, dtype=dtype)
            fields["h1"], fields["h2"] = y, h1
        elif equation == "vti_habc2":
            y, p1 = vti_habc_step(models["vp"], models["epsilon"], models["delta"], fields["p1"], fields["p2"],
                                  dt, h, d, multiple, dtype)
            fields["p1"], fields["p2"] = y, p1
        elif equation == "elastic":
            out = elastic_step(models["vp"], models["vs"], models["rho"],
                               *[fields[n] for n in names], dt, h, d, dtype)
            fields = dict(zip(names, out))
        else:
            raise ValueError(equation)
        wv = dtype(wavelet[i])
        for st in source_type:
            fields[st] = fields[st] + smask * wv
        for b, (zs, xs) in enumerate(receivers):
            zs = np.asarray(zs, int)
            xs = np.asarray(xs, int)
            recs[b].append(np.stack([fields[k][b, zs, xs] for k in receiver_type], axis=-1))
        if illumination:
            illum = illum + np.sum(fields[source_type[-1]] ** 2, axis=0)
    out = {"records": [np.asarray(r) for r in recs], "illum": illum}
    if return_fields:
        out["fields"] = fields
    return out
