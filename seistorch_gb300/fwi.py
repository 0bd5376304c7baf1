"""Full-waveform inversion driver: the plain illumination-preconditioned
method and the learned-preconditioner method, both on the native solver.

Plain: the reference's illumination preconditioning (process.py:115-118),
p = g / (P + eps max P), with Polak-Ribiere conjugate directions (the beta of
optimizer.py:144-224, restarted whenever the direction is not a descent
direction) normalised to max |d| = 1, and a parabolic line search on the data
misfit that uses the known slope g . d at the current model: one trial
step, the minimiser of the parabola through (0, J0) with slope g . d and the
trial, and a shorter step if neither lowers the misfit.

Learned: the network maps [g / max|g|, P / max P] to a model update; the
same line search runs along it, and the update is accepted only if it lowers
the true data misfit, else the plain step is taken -- the misfit stays the
judge of the network's error and the plain method its fallback.

Training pairs come from the solver itself on the inversion's own survey:
random layered + anomaly models, a starting point between the smoothed model
and the truth, and the L2 gradient and source illumination there; the
target is the model error (true - start) / 1000 m/s.
"""
import time

import numpy as np
import torch

from . import engine
from .pml import generate_pml_coefficients_2d
from .postprocess import L2
from .utils import ricker_wave

TARGET_SCALE = 1000.0  # m/s per unit of network output
START_SIGMA = 10.0     # cells: starting models are the true model Gaussian-smoothed by this much


def random_model(rng, nz=256, nx=512, vmin=1500.0, vmax=4500.0):
    """Seeded layered + anomaly velocity model (m/s), nz x nx."""
    zz, xx = np.mgrid[0:nz, 0:nx].astype(np.float64)
    nl = int(rng.integers(3, 8))
    base = np.sort(rng.uniform(0.08, 0.95, nl - 1)) * nz
    vel = np.sort(rng.uniform(vmin, vmax, nl))
    vel[0] = rng.uniform(vmin, vmin + 500.0)
    depth_shift = (rng.uniform(-0.08, 0.08) * (xx - nx / 2)
                   + rng.uniform(0, 12) * np.sin(2 * np.pi * xx / nx * rng.uniform(0.5, 3) + rng.uniform(0, 6)))
    layer = np.zeros((nz, nx), np.int64)
    for k, d in enumerate(base):
        layer += (zz > d + depth_shift).astype(np.int64)
    v = vel[layer]
    for _ in range(int(rng.integers(1, 4))):
        cz, cx = rng.uniform(0.2, 0.9) * nz, rng.uniform(0.1, 0.9) * nx
        r = rng.uniform(8, 35)
        v += rng.choice([-1.0, 1.0]) * rng.uniform(200, 600) * np.exp(-((zz - cz) ** 2 + (xx - cx) ** 2) / (2 * r * r))
    return np.clip(v, vmin, vmax)


def smooth(v, sigma=START_SIGMA):
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(v, sigma, mode="nearest")


class Survey:
    """Acquisition + propagator for inversions on an nz x nx interior grid."""

    def __init__(self, nz=256, nx=512, shots=32, nt=3000, dt=0.001, h=10.0, fm=8.0, width=50, order=4,
                 device=None):
        self.dev = torch.device(device or "cuda")
        self.nzi, self.nxi, self.w = nz, nx, width
        self.nz, self.nx = nz + 2 * width, nx + 2 * width
        self.nt, self.dt, self.h = nt, dt, h
        self.prop = engine.AcousticPropagator(self.nz, self.nx, dt, h, order, "pml", width, False, self.dev)
        xs = np.linspace(0, nx - 1, shots).round().astype(int)
        src = [[(width + 2, width + int(x))] for x in xs]
        rec = [([width + 2] * nx, list(range(width, width + nx)))] * shots
        wav = ricker_wave(fm, dt, nt, delay=int(1.2 / fm / dt), dtype="numpy")
        self.acq = engine.Acquisition(self.nz, self.nx, src, rec, wav, self.dev)
        self.d = generate_pml_coefficients_2d((self.nz, self.nx), width).to(self.dev, torch.float32)
        self.ckpt = engine.default_ckpt_every(nt)

    def pad(self, v):
        """Interior model (numpy or tensor) -> padded device tensor."""
        v = torch.as_tensor(v, dtype=torch.float32, device=self.dev)
        return torch.nn.functional.pad(v[None, None], (self.w,) * 4, mode="replicate")[0, 0].contiguous()

    def records(self, vp_pad):
        with torch.no_grad():
            rec, _ = engine.acoustic_loop(vp_pad, self.prop, self.d, self.acq)
        return rec

    def misfit(self, vp_pad, obs):
        with torch.no_grad():
            return float(L2()(self.records(vp_pad), obs))

    def gradient(self, vp_pad, obs):
        """(misfit, gradient (interior), illumination (interior))."""
        vp = vp_pad.clone().requires_grad_(True)
        rec, illum = engine.acoustic_loop(vp, self.prop, self.d, self.acq, True, self.ckpt)
        loss = L2()(rec, obs)
        loss.backward()
        w = self.w
        return float(loss.detach()), vp.grad[w:-w, w:-w].detach(), illum[w:-w, w:-w].detach()


def features(g, P):
    """Network input [g / max|g|, P / max P] of shape (2, nz, nx)."""
    gn = g / g.abs().max().clamp_min(1e-30)
    pn = P / P.max().clamp_min(1e-30)
    return torch.stack([gn, pn]).to(torch.float32)


def plain_direction(g, P, eps=1e-3):
    d = -g / (P + eps * P.max())
    return d / d.abs().max().clamp_min(1e-30)


def make_pairs(n, survey, seed=0, log=None):
    """n training pairs (features (n, 2, nz, nx), targets (n, nz, nx)) from
    random models, computed by the solver on the device."""
    rng = np.random.default_rng(seed)
    X = torch.empty(n, 2, survey.nzi, survey.nxi, device=survey.dev)
    Y = torch.empty(n, survey.nzi, survey.nxi, device=survey.dev)
    t0 = time.perf_counter()
    for i in range(n):
        vt = random_model(rng, survey.nzi, survey.nxi)
        # a starting model part-way between the smoothed model and the truth,
        # as later inversion iterates are
        tau = rng.uniform(0.0, 0.75) if i % 2 else 0.0
        v0 = smooth(vt)
        v0 = v0 + tau * (vt - v0)
        obs = survey.records(survey.pad(vt))
        _, g, P = survey.gradient(survey.pad(v0), obs)
        X[i] = features(g, P)
        Y[i] = torch.as_tensor((vt - v0) / TARGET_SCALE, dtype=torch.float32, device=survey.dev)
        if log and (i + 1) % 100 == 0:
            log(f"pairs {i + 1}/{n} ({time.perf_counter() - t0:.1f} s)")
    return X, Y


def train(net, X, Y, epochs=10, batch=8, lr=1e-3, seed=0, log=None):
    """Adam on the mean squared error over shuffled mini-batches; returns the
    per-epoch mean loss."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = X.shape[0]
    hist = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g)
        tot = torch.zeros((), device=X.device)
        nb = 0
        lr_ep = lr * (0.5 ** (ep // max(1, epochs // 3)))
        for k in range(0, n - batch + 1, batch):
            idx = perm[k:k + batch].to(X.device)
            tot += net.train_batch(X[idx], Y[idx], lr_ep)[0]
            nb += 1
        hist.append(float(tot) / max(nb, 1))
        if log:
            log(f"epoch {ep + 1}/{epochs}: loss {hist[-1]:.5f}")
    return hist


def line_search(survey, obs, v, J0, g, d, a0, vmin, vmax):
    """Step length along d (max |d| = 1, in m/s) from the misfit J0 with the
    slope s0 = g . d: a trial step a0, then the minimiser of the parabola
    J0 + s0 a + c a^2 through the trial (clipped to [a0/10, 4 a0]), then a
    quarter of the shorter step.  Returns (model, misfit, step) of the best
    step that lowers the misfit, or None."""
    s0 = float((g * d).sum())
    if not s0 < 0:
        return None
    clampv = lambda a: (v + a * d).clamp(vmin, vmax)
    tried = []
    J1 = survey.misfit(survey.pad(clampv(a0)), obs)
    tried.append((J1, a0))
    c = (J1 - J0 - s0 * a0) / (a0 * a0)
    a2 = min(max(-s0 / (2 * c), 0.1 * a0), 4 * a0) if c > 0 else (2 * a0 if J1 < J0 else 0.25 * a0)
    tried.append((survey.misfit(survey.pad(clampv(a2)), obs), a2))
    if min(t[0] for t in tried) >= J0:
        a3 = 0.25 * min(a0, a2)
        tried.append((survey.misfit(survey.pad(clampv(a3)), obs), a3))
    J, a = min(tried)
    if J >= J0:
        return None
    return clampv(a), J, a


def invert(survey, obs, v0, iters=20, net=None, step0=50.0, vmin=1500.0, vmax=4500.0, log=None):
    """FWI from interior model v0.  Returns dict(misfit=[...], time=[...],
    learned_steps=k, model=final interior model).  misfit[i] / time[i]: data
    misfit and elapsed wall time after i iterations (i = 0: start)."""
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    v = torch.as_tensor(v0, dtype=torch.float32, device=survey.dev).clone()
    hist_m, hist_t = [], []
    learned_steps = 0
    J, g, P = survey.gradient(survey.pad(v), obs)
    hist_m.append(J)
    hist_t.append(time.perf_counter() - t0)
    p_prev = d_prev = None
    a_plain, a_net = step0, 1.0
    for it in range(iters):
        res = None
        if net is not None:
            dv = net.predict(features(g, P)[None])[0] * TARGET_SCALE
            scale = float(dv.abs().max().clamp_min(1e-30))
            res = line_search(survey, obs, v, J, g, dv / scale, a_net * scale, vmin, vmax)
            if res is not None:
                a_net = res[2] / scale
                learned_steps += 1
                p_prev = d_prev = None  # the conjugate directions restart after a learned step
        if res is None:
            p = g / (P + 1e-3 * P.max())
            d = -p
            if p_prev is not None:
                beta = float(((p - p_prev) * p).sum() / (p_prev * p_prev).sum().clamp_min(1e-30))
                d = -p + max(beta, 0.0) * d_prev
                if not float((g * d).sum()) < 0:
                    d = -p
            d = d / d.abs().max().clamp_min(1e-30)
            res = line_search(survey, obs, v, J, g, d, a_plain, vmin, vmax)
            if res is None and p_prev is not None:  # restart along the preconditioned gradient
                d = -p / p.abs().max().clamp_min(1e-30)
                res = line_search(survey, obs, v, J, g, d, a_plain, vmin, vmax)
            p_prev, d_prev = p, d
            if res is not None:
                a_plain = res[2]
            else:
                a_plain *= 0.25
        if res is not None:
            v = res[0]
        J, g, P = survey.gradient(survey.pad(v), obs)
        hist_m.append(J)
        torch.cuda.synchronize()
        hist_t.append(time.perf_counter() - t0)
        if log:
            log(f"iter {it + 1}: misfit {J:.4e} ({hist_t[-1]:.1f} s)")
    return {"misfit": hist_m, "time": hist_t, "learned_steps": learned_steps, "model": v}
