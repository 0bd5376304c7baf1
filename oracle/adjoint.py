"""Exact discrete adjoints of the oracle time loops (gradient oracle).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

The reference obtains model gradients by autograd through every step of
``WaveRNN.forward`` (rnn.py:178-205, ``boundary_saving: false``).  These
functions compute the same quantity by the transposed recursions, keeping
every forward state in memory (small cases only).  ``record_grads[b]`` is
dJ/d(records of shot b), shape (nt, nrec_b, nch); for the L2 misfit
(loss.py:409-421) it is 2*(syn - obs).
"""
import numpy as np

from . import fd2d


def _inject(fields, b, zs, xs, vals):
    np.add.at(fields[b], (np.asarray(zs, int), np.asarray(xs, int)), vals)


def acoustic_pml_gradient(vp, d, dt, h, wavelet, sources, receivers, record_grads, order=2,
                          dtype=np.float64, keep_every=None):
    """dJ/dvp for the 2nd-order acoustic PML loop (acoustic.py:73-86).

    Forward: U_{i+1} = A U_i - Bc U_{i-1} + Kv Lh(U_i) + S w_i with
    inv = (dt^-2 + d/dt)^-1, A = 2 inv/dt^2, Bc = inv (dt^-2 - d/dt),
    Kv = inv vp^2; records r_i = R U_{i+1}.
    Adjoint (Lh is self-adjoint, zero padded):
      lam_k = R^T g_{k-1} + A lam_{k+1} + Lh(Kv lam_{k+1}) - Bc lam_{k+2}
    Gradient: dJ/dvp = sum_i lam_{i+1} * 2 vp inv * Lh(U_i).
    Every forward state is kept by default; with ``keep_every = S`` only
    the pairs (U_{a-1}, U_a) at a = 0, S, 2S, ... are kept and each segment
    is recomputed in the reverse sweep (the same float64 arithmetic, so the
    result is identical), which bounds memory for long runs.
    """
    vp = np.asarray(vp, dtype)
    d = np.asarray(d, dtype)
    dt = dtype(dt)
    nt = len(wavelet)
    B = len(sources)
    nz, nx = vp.shape
    inv = dtype(1.0) / (dt ** -2 + d / dt)
    A = dtype(2.0) * inv / dt ** 2
    Bc = inv * (dt ** -2 - d / dt)
    Kv = inv * vp ** 2
    smask = np.zeros((B, nz, nx), dtype)
    for b, pts in enumerate(sources):
        for (z, x) in pts:
            smask[b, z, x] = 1

    def step(um1, u0, i):
        y = A * u0 - Bc * um1 + Kv * fd2d.laplacian(u0, order, h, dtype)
        return y + smask * dtype(np.float32(wavelet[i]))

    zero = np.zeros((B, nz, nx), dtype)
    if keep_every is None:
        U = [zero, zero]  # U_{-1}, U_0
        for i in range(nt):
            U.append(step(U[-2], U[-1], i))

        def states_reversed():  # U_{nt-1}, ..., U_0
            for m in range(nt - 1, -1, -1):
                yield U[m + 1]
    else:
        S = int(keep_every)
        ck = {}
        prev, cur = zero, zero
        for i in range(nt):
            if i % S == 0:
                ck[i] = (prev, cur)  # (U_{i-1}, U_i)
            prev, cur = cur, step(prev, cur, i)

        def states_reversed():
            for a in sorted(ck, reverse=True):
                um1, u0 = ck[a]
                seg = [u0]
                for i in range(a, min(a + S, nt) - 1):
                    um1, u0 = u0, step(um1, u0, i)
                    seg.append(u0)
                yield from reversed(seg)

    states = states_reversed()
    grad = np.zeros((nz, nx), dtype)
    lam1 = np.zeros((B, nz, nx), dtype)   # lam_{k+1}
    lam2 = np.zeros((B, nz, nx), dtype)   # lam_{k+2}
    for k in range(nt, 0, -1):
        lam = A * lam1 + fd2d.laplacian(Kv * lam1, order, h, dtype) - Bc * lam2
        for b, (zs, xs) in enumerate(receivers):
            _inject(lam, b, zs, xs, np.asarray(record_grads[b][k - 1][:, 0], dtype))
        # term i = k-1: lam_k * dU_k/dvp = lam_k * 2 vp inv Lh(U_{k-1})
        grad += np.sum(lam * fd2d.laplacian(next(states), order, h, dtype), axis=0)
        lam2, lam1 = lam1, lam
    return grad * dtype(2.0) * vp * inv


def _dfwd_T(g, axis):
    """Transpose of ``fd2d.dfwd`` (a[i]-a[i-1], zero at i=0)."""
    out = np.array(g, copy=True)
    n = g.shape[axis]
    sl = [slice(None)] * g.ndim
    sl[axis] = 0
    out[tuple(sl)] = 0
    a = [slice(None)] * g.ndim
    bsl = [slice(None)] * g.ndim
    a[axis] = slice(0, n - 1)
    bsl[axis] = slice(1, n)
    out[tuple(a)] -= g[tuple(bsl)]
    return out


def _dbwd_T(g, axis):
    """Transpose of ``fd2d.dbwd`` (a[i+1]-a[i], zero at i=n-1)."""
    n = g.shape[axis]
    out = np.zeros_like(g)
    a = [slice(None)] * g.ndim
    bsl = [slice(None)] * g.ndim
    a[axis] = slice(1, n)
    bsl[axis] = slice(0, n - 1)
    out[tuple(a)] += g[tuple(bsl)]
    out[tuple(bsl)] -= g[tuple(bsl)]
    return out


def elastic_gradient(vp, vs, rho, d, dt, h, wavelet, sources, receivers, record_grads,
                     source_type=("txx", "tzz"), receiver_type=("vx", "vz")):
    """dJ/d(vp, vs, rho) for the velocity-stress loop (elastic.py:7-37).

    Forward step (a = (1-c)/(1+c), e = dt/(h(1+c)), bu = dt/(rho h (1+c))):
      sxx'' = a sxx + e (P Dx- vx + L Dz+ vz),  szz'' = a szz + e (P Dz+ vz + L Dx- vx)
      sxz'' = a sxz + e M (Dx+ vz + Dz- vx)
      vx'   = a vx + bu (Dx+ sxx'' + Dz+ sxz''),  vz' = a vz + bu (Dx- sxz'' + Dz- szz'')
    then sources add to the stresses; receivers read vx', vz'.  With
    P = L + 2M, L = rho (vp^2 - 2 vs^2), M = rho vs^2.
    """
    vp, vs, rho, d = (np.asarray(x, np.float64) for x in (vp, vs, rho, d))
    nt = len(wavelet)
    B = len(sources)
    nz, nx = vp.shape
    c = 0.5 * dt * d
    a = (1 - c) / (1 + c)
    e = dt / h / (1 + c)
    bu = dt / rho / h / (1 + c)
    Lm = rho * (vp ** 2 - 2 * vs ** 2)
    Mu = rho * vs ** 2
    P = Lm + 2 * Mu
    names = ["vx", "vz", "txx", "tzz", "txz"]
    smask = np.zeros((B, nz, nx))
    for b, pts in enumerate(sources):
        for (z, x) in pts:
            smask[b, z, x] = 1
    states = [{n: np.zeros((B, nz, nx)) for n in names}]
    mids = []
    for i in range(nt):
        s = states[-1]
        ax = fd2d.dfwd(s["vx"], 2)
        bz = fd2d.dbwd(s["vz"], 1)
        sxx = a * s["txx"] + e * (P * ax + Lm * bz)
        szz = a * s["tzz"] + e * (P * bz + Lm * ax)
        sxz = a * s["txz"] + e * Mu * (fd2d.dbwd(s["vz"], 2) + fd2d.dfwd(s["vx"], 1))
        vx = a * s["vx"] + bu * (fd2d.dbwd(sxx, 2) + fd2d.dbwd(sxz, 1))
        vz = a * s["vz"] + bu * (fd2d.dfwd(sxz, 2) + fd2d.dfwd(szz, 1))
        mids.append((sxx, szz, sxz))
        new = {"vx": vx, "vz": vz, "txx": sxx, "tzz": szz, "txz": sxz}
        w = np.float64(np.float32(wavelet[i]))
        for st in source_type:
            new[st] = new[st] + smask * w
        states.append(new)
    g_P = np.zeros((nz, nx))
    g_L = np.zeros((nz, nx))
    g_M = np.zeros((nz, nx))
    g_bu = np.zeros((nz, nx))
    adj = {n: np.zeros((B, nz, nx)) for n in names}
    for i in range(nt - 1, -1, -1):
        for b, (zs, xs) in enumerate(receivers):
            for ch, key in enumerate(receiver_type):
                _inject(adj[key], b, zs, xs, record_grads[b][i][:, ch])
        s = states[i]
        sxx, szz, sxz = mids[i]
        avx, avz = adj["vx"], adj["vz"]
        g_bu += np.sum(avx * (fd2d.dbwd(sxx, 2) + fd2d.dbwd(sxz, 1))
                       + avz * (fd2d.dfwd(sxz, 2) + fd2d.dfwd(szz, 1)), axis=0)
        a_sxx = adj["txx"] + _dbwd_T(bu * avx, 2)
        a_sxz = adj["txz"] + _dbwd_T(bu * avx, 1) + _dfwd_T(bu * avz, 2)
        a_szz = adj["tzz"] + _dfwd_T(bu * avz, 1)
        ax = fd2d.dfwd(s["vx"], 2)
        bz = fd2d.dbwd(s["vz"], 1)
        shear = fd2d.dbwd(s["vz"], 2) + fd2d.dfwd(s["vx"], 1)
        g_P += np.sum(e * (a_sxx * ax + a_szz * bz), axis=0)
        g_L += np.sum(e * (a_sxx * bz + a_szz * ax), axis=0)
        g_M += np.sum(e * a_sxz * shear, axis=0)
        alpha = e * (P * a_sxx + Lm * a_szz)
        beta = e * (Lm * a_sxx + P * a_szz)
        gam = e * Mu * a_sxz
        adj = {"vx": a * avx + _dfwd_T(alpha, 2) + _dfwd_T(gam, 1),
               "vz": a * avz + _dbwd_T(beta, 1) + _dbwd_T(gam, 2),
               "txx": a * a_sxx, "tzz": a * a_szz, "txz": a * a_sxz}
    g_lam = g_P + g_L
    g_mu = 2 * g_P + g_M
    grad_vp = g_lam * 2 * rho * vp
    grad_vs = g_lam * (-4 * rho * vs) + g_mu * 2 * rho * vs
    grad_rho = g_lam * (vp ** 2 - 2 * vs ** 2) + g_mu * vs ** 2 - g_bu * bu / rho
    return grad_vp, grad_vs, grad_rho
